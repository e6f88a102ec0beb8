// Multiscale cascade detection on sm_103a, for one image (vj_detect, the
// drop-in for FaceVisionEngine::detectMultiScale, src/face_vision_engine.cu:
// 1541-1747) or many images at once (vj_detect_batch).
//
// Every call runs one persistent cooperative kernel (cascade.cuh) over all
// pyramid levels of all its images, replayed from a CUDA graph that this
// detector captures once: [plan H2D] -> [control-block memset] -> [kernel] ->
// [control-block D2H].  The kernel reads everything about the batch from the
// device-resident plan (levels, resize chain, integral jobs, stage schedule,
// buffer pointers), so the same graph serves every batch; only the size of
// the plan copy is updated per launch.  The raw detections arrive in a
// host-mapped buffer, so the host waits once per call.
//
// The host then sorts each image's raw detections into the reference CPU
// path's order (level, y, x), truncates to maxDetections and groups them
// (groupRectangles, face_vision_engine.cu:1401-1539).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "cascade.cuh"
#include "group.h"
#include "launch_chain.h"

namespace vjgb {
namespace {

// Device buffer: owned and grown on demand, or (view) a fixed range of the
// detector's arena, which never grows.
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    bool view = false;
    // Grows to at least `bytes`; returns VJ_OK.  Contents are not kept.
    int ensure(size_t bytes) {
        if (bytes <= cap && p) return VJ_OK;
        if (view) return set_error(VJ_OUT_OF_MEMORY, "detector arena: batch does not fit the reserved bytes");
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 8, 256);
        const cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return set_error(e == cudaErrorMemoryAllocation ? VJ_OUT_OF_MEMORY : VJ_CUDA_ERROR,
                             std::string("detector buffer: ") + cudaGetErrorString(e));
        }
        cap = want;
        return VJ_OK;
    }
    void release() {
        if (p && !view) cudaFree(p);
        p = nullptr;
        cap = 0;
        view = false;
    }
    void set_view(void* base, size_t bytes) {
        release();
        p = base;
        cap = bytes;
        view = true;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

// Pinned host buffer; `mapped` ones are also addressable by kernels.
struct HBuf {
    void* p = nullptr;
    void* dev = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes, bool mapped = false) {
        if (bytes <= cap && p) return VJ_OK;
        if (p) cudaFreeHost(p);
        p = dev = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 8, 256);
        cudaError_t e = cudaHostAlloc(&p, want, mapped ? cudaHostAllocMapped : cudaHostAllocDefault);
        if (e == cudaSuccess && mapped) e = cudaHostGetDevicePointer(&dev, p, 0);
        if (e != cudaSuccess) {
            if (p) cudaFreeHost(p);
            p = dev = nullptr;
            return set_error(VJ_OUT_OF_MEMORY, std::string("pinned buffer: ") + cudaGetErrorString(e));
        }
        cap = want;
        return VJ_OK;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = dev = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct LevelGeom {
    int scaleIdx;
    float scale;
    int w, h, step;
    int src;  // index of the level it is resized from in this image's list; -2 = the image itself
};

// Level schedule of detectMultiScale (face_vision_engine.cu:1589-1713): scale
// grows by fp32 multiplication; level sizes round(W / scale); levels whose
// object size is below minObjectSize are skipped without resizing; the loop
// stops when a level is smaller than the window.
std::vector<LevelGeom> plan_levels(int W, int H, int winW, int winH, float sf, int minObj) {
    std::vector<LevelGeom> out;
    float scale = 1.0f;
    int idx = 0, prev = -1;
    for (;;) {
        const int sw = static_cast<int>(std::round(static_cast<float>(W) / scale));
        const int sh = static_cast<int>(std::round(static_cast<float>(H) / scale));
        const int ow = static_cast<int>(std::round(static_cast<float>(winW) * scale));
        const int oh = static_cast<int>(std::round(static_cast<float>(winH) * scale));
        if (sw < winW || sh < winH) break;
        if (!(ow < minObj || oh < minObj)) {
            LevelGeom g;
            g.scaleIdx = idx;
            g.scale = scale;
            g.w = sw;
            g.h = sh;
            g.step = (scale >= 3.0f) ? 3 : ((scale >= 2.0f) ? 2 : 1);
            g.src = idx == 0 ? -2 : prev;
            out.push_back(g);
            prev = static_cast<int>(out.size()) - 1;
        }
        scale *= sf;
        ++idx;
        if (idx > 100000) break;
    }
    return out;
}

int sm_count() {
    static int c = 0;
    if (!c) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        c = v > 0 ? v : 1;
    }
    return c;
}

inline int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool canonical_less(const vj_detection& a, const vj_detection& b) {
    if (a.scaleIdx != b.scaleIdx) return a.scaleIdx < b.scaleIdx;
    if (a.y != b.y) return a.y < b.y;
    return a.x < b.x;
}

}  // namespace

}  // namespace vjgb

using namespace vjgb;

struct vj_detector {
    int winW = 24, winH = 24, maxW = 0, maxH = 0, maxDet = 0;
    int normMode = VJ_NORM_FLOAT_CORNERS;
    int nStages = 0, nStumps = 0;
    std::vector<DStage> hStages;
    DBuf stumps, pstumps, stages;  // pstumps: planes A, B, C of nStumps uint4 each
    bool spreadStumps = false;     // the planes are reordered within blocks (spread_banks)
    // Work buffers, grown on demand.
    DBuf imgs, pix, iiSum, iiSq, totS, totQ, qA, qB, dets, dplan, dctrl, ghist;
    HBuf hplan, hctrl, hdets;
    HBuf himgs;  // pinned staging of a large batch's host images, laid out as `imgs`
    int imageCap = 0;  // images the control block has room for
    // Optional arena (vj_detector_reserve): every work buffer of a batch is a
    // range of it, so the detector never holds more than its reservation.
    DBuf arena;
    // Launch shape and the stage schedule derived from it.
    vj_detect_config cfg{8, 64, 0, 0, 2, 0};
    int tileStages = 0, deepFrom = 0;
    std::vector<int> queueEnds;
    // Launch graph and what it was built for.
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t planNode = nullptr;
    int graphTH = 0, graphGrid = 0, graphBps = 0;
    size_t graphPlanBytes = 0;  // size the plan copy node was last given
    const void* graphFn = nullptr;
    size_t graphSmem = 0, graphCtrlBytes = 0;
    void* graphPlan = nullptr;
    void* graphCtrl = nullptr;
    void* graphHCtrl = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // Capacity hints: the largest queue, per-image raw count and total raw
    // count seen so far, so a repeated workload needs no retry.
    int64_t qHint = 0;
    int detHint = 0;
    int64_t hostHint = 0;
    int64_t grpHint = 0;  // kept raw detections of a grouped call
    vj_detect_stats stats{};
    // Wait test (vj_detector_test_barrier_timeout): one block leaves before
    // the first grid barrier and the others wait at most this long.
    int testHoldBlock = -1;
    unsigned long long testBarrierTimeoutNs = 0;
    LaunchChain* chain = nullptr;  // launch ordering shared with other detectors
};

namespace {

void drop_graph(vj_detector* d) {
    if (d->exec) cudaGraphExecDestroy(d->exec);
    if (d->graph) cudaGraphDestroy(d->graph);
    d->exec = nullptr;
    d->graph = nullptr;
    d->planNode = nullptr;
    d->graphTH = 0;
}

// Stage schedule: the tile pass runs whole stages until it has covered
// cfg.tileStumps stumps; queue passes (at most kMaxQueuePasses) then cover at
// least cfg.queueStumps more, split evenly; the deep pass takes the rest.
void schedule_passes(vj_detector* d) {
    int acc = 0, s = 0;
    while (s < d->nStages && (acc < d->cfg.tileStumps || s == 0)) acc += d->hStages[s++].ntrees;
    d->tileStages = s;
    d->queueEnds.clear();
    if (d->cfg.queueStumps > 0 && s < d->nStages) {
        int target = 0, total = 0;
        const int s0 = s;
        while (s < d->nStages && target < d->cfg.queueStumps) target += d->hStages[s++].ntrees;
        s = s0;
        const int per = std::max(1, (target + kMaxQueuePasses - 1) / kMaxQueuePasses);
        while (s < d->nStages && total < target) {
            int a = 0;
            while (s < d->nStages && a < per && total + a < target) a += d->hStages[s++].ntrees;
            total += a;
            d->queueEnds.push_back(s);
            if (static_cast<int>(d->queueEnds.size()) == kMaxQueuePasses) break;
        }
    }
    d->deepFrom = d->queueEnds.empty() ? d->tileStages : d->queueEnds.back();
}

template <int TH, int SL>
const void* kernel_for(int blocksPerSM) {
    if (blocksPerSM >= 4) return reinterpret_cast<const void*>(&detect_persistent_kernel<TH, 4, SL>);
    return reinterpret_cast<const void*>(&detect_persistent_kernel<TH, 3, SL>);
}

template <int TH>
const void* kernel_for_slots(int blocksPerSM, int slots) {
    return slots == 1 ? kernel_for<TH, 1>(blocksPerSM) : kernel_for<TH, 2>(blocksPerSM);
}

// Kernel variant for a launch shape: tile rows, deep-pass window slots, and
// the residency the kernel is compiled for - 3 (blocksPerSM 0-3) or 4 CTAs of
// 256 threads per SM, which caps its registers at 85 or 64.
const void* kernel_ptr(const vj_detect_config& c) {
    switch (c.tileRows) {
        case 4: return kernel_for_slots<4>(c.blocksPerSM, c.deepSlots);
        case 16: return kernel_for_slots<16>(c.blocksPerSM, c.deepSlots);
        default: return kernel_for_slots<8>(c.blocksPerSM, c.deepSlots);
    }
}

size_t smem_bytes(const vj_detector* d, int th) {
    const size_t lists = static_cast<size_t>(kCasWarps) * 32 * th * sizeof(uint2);  // cascade.cuh lane_pass
    const size_t deep = static_cast<size_t>(kCasWarps) *
                        deep_warp_floats(d->cfg.deepSlots, (d->winW + 1) * (d->winH + 1)) * sizeof(float);
    return std::max(lists, deep);
}

// Control block: CtrlHead, then int counts, offsets, rawOff, ccount and
// gcount[imageCap], then uint64 selKey[imageCap].
constexpr int kCtrlIntArrays = 5;
size_t ctrl_sel_offset(int imageCap) {
    return align_up(align_up(sizeof(CtrlHead), 16) + kCtrlIntArrays * sizeof(int) * static_cast<size_t>(imageCap), 16);
}
size_t ctrl_bytes(int imageCap) { return ctrl_sel_offset(imageCap) + sizeof(uint64_t) * static_cast<size_t>(imageCap); }

// Grouping slots the two queue buffers hold (group_dev.cuh: kGroupBytesA/B
// per slot, plus alignment).
int64_t group_slots(size_t qaBytes, size_t qbBytes) {
    const int64_t a = (static_cast<int64_t>(qaBytes) - 16 * 256) / kGroupBytesA;
    const int64_t b = (static_cast<int64_t>(qbBytes) - 16 * 256) / kGroupBytesB;
    return std::max<int64_t>(0, std::min<int64_t>({a, b, INT32_MAX / 2}));
}

// Carves the grouping arrays of `cap` slots from the queue buffers.
void carve_group(GroupPlan& g, char* qa, char* qb, int cap) {
    size_t o = 0;
    auto take = [&o](char* base, size_t bytes) {
        o = static_cast<size_t>(align_up(static_cast<int64_t>(o), 256));
        char* p = base + o;
        o += bytes;
        return p;
    };
    const size_t n = static_cast<size_t>(cap);
    g.key = reinterpret_cast<unsigned long long*>(take(qa, 8 * n));
    g.x = reinterpret_cast<int*>(take(qa, 4 * n));
    g.y = reinterpret_cast<int*>(take(qa, 4 * n));
    g.w = reinterpret_cast<int*>(take(qa, 4 * n));
    g.h = reinterpret_cast<int*>(take(qa, 4 * n));
    g.score = reinterpret_cast<float*>(take(qa, 4 * n));
    g.parent = reinterpret_cast<int*>(take(qa, 4 * n));
    g.root = reinterpret_cast<int*>(take(qa, 4 * n));
    g.image = reinterpret_cast<int*>(take(qa, 4 * n));
    o = 0;
    g.sumX = reinterpret_cast<unsigned long long*>(take(qb, 8 * n));
    g.sumY = reinterpret_cast<unsigned long long*>(take(qb, 8 * n));
    g.sumW = reinterpret_cast<unsigned long long*>(take(qb, 8 * n));
    g.sumH = reinterpret_cast<unsigned long long*>(take(qb, 8 * n));
    g.bestKey = reinterpret_cast<unsigned long long*>(take(qb, 8 * n));
    g.cl = reinterpret_cast<GCluster*>(take(qb, sizeof(GCluster) * n));
    g.cnt = reinterpret_cast<int*>(take(qb, 4 * n));
    g.best = reinterpret_cast<unsigned*>(take(qb, 4 * n));
    g.order = reinterpret_cast<int*>(take(qb, 4 * n));
}

// Builds (or rebuilds) the launch graph for the current launch shape and
// plan/control buffers.
int ensure_graph(vj_detector* d, size_t planBytes) {
    const int th = d->cfg.tileRows;
    const size_t smem = smem_bytes(d, th);
    const size_t cbytes = ctrl_bytes(d->imageCap);
    const void* fn = kernel_ptr(d->cfg);
    // set on every call: detectors with other window sizes share the kernel
    VJ_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    // the grid follows from (kernel, shared memory, blocksPerSM): a graph
    // built for the same ones and buffers is replayed without asking again
    if (d->exec && d->graphFn == fn && d->graphTH == th && d->graphBps == d->cfg.blocksPerSM &&
        d->graphSmem == smem && d->graphPlan == d->dplan.p && d->graphCtrl == d->dctrl.p &&
        d->graphCtrlBytes == cbytes && d->graphHCtrl == d->hctrl.p)
        return VJ_OK;
    int fit = 0;
    VJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, kCasThreads, smem));
    if (fit < 1) return set_error(VJ_RUNTIME_ERROR, "detection kernel does not fit on an SM");
    const int bps = d->cfg.blocksPerSM > 0 ? std::min(d->cfg.blocksPerSM, fit) : fit;
    const int grid = bps * sm_count();
    drop_graph(d);
    cudaGraph_t g = nullptr;
    VJ_CUDA_TRY(cudaGraphCreate(&g, 0));
    auto fail = [&](cudaError_t e, const char* what) {
        cudaGraphDestroy(g);
        return set_error(VJ_CUDA_ERROR, std::string("detection graph: ") + what + ": " + cudaGetErrorString(e));
    };
    cudaGraphNode_t nPlan, nSet, nKer, nBack;
    cudaError_t e = cudaGraphAddMemcpyNode1D(&nPlan, g, nullptr, 0, d->dplan.p, d->hplan.p, planBytes,
                                             cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(e, "plan copy node");
    cudaMemsetParams mp{};
    mp.dst = d->dctrl.p;
    mp.value = 0;
    mp.elementSize = 1;
    mp.width = cbytes;
    mp.height = 1;
    mp.pitch = 0;
    e = cudaGraphAddMemsetNode(&nSet, g, &nPlan, 1, &mp);
    if (e != cudaSuccess) return fail(e, "control memset node");
    void* planArg = d->dplan.p;
    void* args[] = {&planArg};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(fn);
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(kCasThreads);
    kp.sharedMemBytes = static_cast<unsigned>(smem);
    kp.kernelParams = args;
    kp.extra = nullptr;
    e = cudaGraphAddKernelNode(&nKer, g, &nSet, 1, &kp);
    if (e != cudaSuccess) return fail(e, "kernel node");
    cudaLaunchAttributeValue coop{};
    coop.cooperative = 1;
    e = cudaGraphKernelNodeSetAttribute(nKer, cudaLaunchAttributeCooperative, &coop);
    if (e != cudaSuccess) return fail(e, "cooperative attribute");
    e = cudaGraphAddMemcpyNode1D(&nBack, g, &nKer, 1, d->hctrl.p, d->dctrl.p, cbytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(e, "control copy node");
    cudaGraphExec_t x = nullptr;
    e = cudaGraphInstantiate(&x, g, 0);
    if (e != cudaSuccess) return fail(e, "instantiate");
    d->graph = g;
    d->exec = x;
    d->planNode = nPlan;
    d->graphTH = th;
    d->graphFn = fn;
    d->graphGrid = grid;
    d->graphBps = d->cfg.blocksPerSM;
    d->graphPlanBytes = planBytes;
    d->graphSmem = smem;
    d->graphCtrlBytes = cbytes;
    d->graphPlan = d->dplan.p;
    d->graphCtrl = d->dctrl.p;
    d->graphHCtrl = d->hctrl.p;
    return VJ_OK;
}

struct BatchImage {
    const uint8_t* ptr;
    int w, h;
    int64_t stride;
};

constexpr int64_t kStageImageBytes = int64_t(16) << 20;

// Copies the rows of the images not read in place (skip[i] null) into `dst`
// at pitch align_up(w, 16) from offset off[i], on up to 16 host threads
// taking blocks of about 2 MB of rows.
void stage_images(const std::vector<BatchImage>& ims, const std::vector<int64_t>& off,
                  const std::vector<const uint8_t*>& skip, uint8_t* dst) {
    struct Piece {
        int img, r0, r1;
    };
    std::vector<Piece> pieces;
    for (int i = 0; i < static_cast<int>(ims.size()); ++i) {
        if (skip[i]) continue;
        const int rowsPer = std::max(1, static_cast<int>((int64_t(2) << 20) / std::max(1, ims[i].w)));
        for (int r = 0; r < ims[i].h; r += rowsPer) pieces.push_back({i, r, std::min(ims[i].h, r + rowsPer)});
    }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t k; (k = next.fetch_add(1)) < pieces.size();) {
            const Piece& pc = pieces[k];
            const BatchImage& im = ims[pc.img];
            const int64_t pitch = align_up(static_cast<int64_t>(im.w), 16);
            uint8_t* d = dst + off[pc.img] + pitch * pc.r0;
            const uint8_t* src = im.ptr + im.stride * pc.r0;
            if (im.stride == pitch) {
                std::memcpy(d, src, static_cast<size_t>(pitch) * (pc.r1 - pc.r0 - 1) + im.w);
            } else {
                for (int r = pc.r0; r < pc.r1; ++r, d += pitch, src += im.stride) std::memcpy(d, src, im.w);
            }
        }
    };
    const int T = static_cast<int>(std::min<size_t>(
        pieces.size(), std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 1; t < T; ++t) th.emplace_back(work);
    work();
    for (auto& x : th) x.join();
}

// Grouping on the device: off, or on with groupRectangles' minNeighbors and
// the per-image raw detection limit.
struct GroupArgs {
    bool on = false;
    int minN = 0;
    int limit = 0;
};

// Runs the detection kernel over `ims`.  On return, without grouping, the raw
// detections of image i are hdets[offsets[i] .. offsets[i] + min(counts[i],
// detCap)); with grouping its grouped detections are hdets[offsets[i] ..
// offsets[i] + grouped[i]) in cluster order.
int execute(vj_detector* D, const std::vector<BatchImage>& ims, bool onDevice, float sf, int minObj,
            const GroupArgs& ga, cudaStream_t s, const int** outCounts, const int** outOffsets, int* outDetCap,
            const int** outGrouped = nullptr) {
    const int nImg = static_cast<int>(ims.size());
    const double t0 = now_ms();
    // ---- levels and sizes
    std::vector<std::vector<LevelGeom>> geo(nImg);
    int64_t pixBytes = 0, iiElems = 0, imgBytes = 0;
    // Host images.  When the page-locked images of the call add up to
    // kStageImageBytes or more, the kernel reads each of them in place through
    // its mapped device address (over the host link; no copy).  The others
    // reach the device at a 16-byte pitch (the integral row pass reads 16
    // pixels per load): an image whose rows are already at that pitch, or a
    // page-locked one whose stride is a multiple of 16 (and below w + 64), is
    // one contiguous copy at its own stride; the rest go at pitch
    // align_up(w, 16), row by row, unless the copied images add up to
    // kStageImageBytes or more: then host threads gather them into a pinned
    // buffer in the device layout, moved by one copy (row by row copies of 256
    // scenes moved about 16 GB/s).
    std::vector<int64_t> imgOff(nImg, 0), imgPitch(nImg, 0);
    std::vector<char> dense(nImg, 0);
    std::vector<const uint8_t*> mapped(nImg, nullptr);
    std::vector<char> locked(nImg, 0);
    bool staged = false;
    if (!onDevice) {
        int64_t rowwise = 0, lockedBytes = 0;
        for (int i = 0; i < nImg; ++i) {
            cudaPointerAttributes a{};
            locked[i] = cudaPointerGetAttributes(&a, ims[i].ptr) == cudaSuccess && a.type == cudaMemoryTypeHost;
            if (!locked[i]) cudaGetLastError();
            if (locked[i] && a.devicePointer) {
                mapped[i] = static_cast<const uint8_t*>(a.devicePointer);
                lockedBytes += ims[i].stride * ims[i].h;
            }
        }
        if (lockedBytes < kStageImageBytes) std::fill(mapped.begin(), mapped.end(), nullptr);
        for (int i = 0; i < nImg; ++i) {
            if (mapped[i]) continue;
            dense[i] = (locked[i] && ims[i].stride % 16 == 0 && ims[i].stride < ims[i].w + 64) ||
                       ims[i].stride == align_up(static_cast<int64_t>(ims[i].w), 16);
            if (!dense[i]) rowwise += align_up(static_cast<int64_t>(ims[i].w), 16) * ims[i].h;
        }
        staged = rowwise >= kStageImageBytes;
        if (staged) std::fill(dense.begin(), dense.end(), 0);
    }
    for (int i = 0; i < nImg; ++i) {
        geo[i] = plan_levels(ims[i].w, ims[i].h, D->winW, D->winH, sf, minObj);
        if (!onDevice && !mapped[i]) {
            imgOff[i] = imgBytes;
            imgPitch[i] = dense[i] ? ims[i].stride : align_up(static_cast<int64_t>(ims[i].w), 16);
            const int64_t bytes = ims[i].h <= 0 ? 0
                                  : dense[i] ? imgPitch[i] * (ims[i].h - 1) + ims[i].w
                                             : imgPitch[i] * ims[i].h;
            imgBytes += align_up(bytes, 16);
        }
        for (const auto& g : geo[i]) {
            if (g.src != -2) pixBytes += align_up(g.w, 16) * g.h;
            iiElems += (g.h + 1) * ii_pitch(g.w);
        }
    }
    int64_t totRows = 0, totPitch = 0, walkItems = 0, windowsAll = 0;
    for (int i = 0; i < nImg; ++i)
        for (const auto& g : geo[i]) {
            totRows += col_segs(g.h);
            totPitch = std::max<int64_t>(totPitch, static_cast<int64_t>(col_chunks(g.w)) * 32);
            walkItems += col_chunks(g.w);
            windowsAll += static_cast<int64_t>((g.w - D->winW + g.step) / g.step) * ((g.h - D->winH + g.step) / g.step);
        }
    // Column pass of the integrals: one walk per 32-column chunk down all
    // rows when there are enough chunks to keep every warp of the grid busy
    // several times over (16 B per element moved), else segment totals and a
    // segment scan (32-row segments, enough items for any image; 24 B per
    // element and a grid barrier more).
    const int64_t gridWarps = static_cast<int64_t>(sm_count()) * 3 * kCasWarps;
    const bool colWalk = walkItems >= 4 * gridWarps;
    const int64_t totElems = colWalk ? 1 : std::max<int64_t>(1, totRows * totPitch);
    // the grouping arrays reuse the queue buffers after the deep pass
    const int64_t grpQ = ga.on ? (D->grpHint * kGroupBytesB + 16 * 256) / static_cast<int64_t>(sizeof(QEntry)) + 1 : 0;
    int64_t qcap =
        std::min<int64_t>(std::max<int64_t>({windowsAll / 8, int64_t(1) << 16, D->qHint, grpQ}), INT32_MAX / 2);
    std::vector<int64_t> histBase(static_cast<size_t>(nImg) + 1, 0);
    for (int i = 0; i < nImg; ++i) histBase[i + 1] = histBase[i] + ims[i].w + 1;
    const int64_t histTotal = ga.on ? histBase[nImg] : 0;
    int detCap = std::max({64, std::min(D->maxDet, 4096), D->detHint});
    // Work buffers: grown on demand, or carved from the arena with the queues
    // taking whatever the other buffers leave.
    auto layout = [&]() -> int {
        const size_t detBytes = sizeof(vj_detection) * static_cast<size_t>(detCap) * nImg;
        if (!D->arena.p) {
            int r;
            if (!onDevice && (r = D->imgs.ensure(imgBytes)) != VJ_OK) return r;
            if ((r = D->pix.ensure(pixBytes)) != VJ_OK) return r;
            if ((r = D->iiSum.ensure(iiElems * 4)) != VJ_OK) return r;
            if ((r = D->iiSq.ensure(iiElems * 4)) != VJ_OK) return r;
            if ((r = D->totS.ensure(totElems * 4)) != VJ_OK) return r;
            if ((r = D->totQ.ensure(totElems * 4)) != VJ_OK) return r;
            if ((r = D->dets.ensure(detBytes)) != VJ_OK) return r;
            if (histTotal && (r = D->ghist.ensure(static_cast<size_t>(histTotal) * 4)) != VJ_OK) return r;
            if ((r = D->qA.ensure(sizeof(QEntry) * static_cast<size_t>(qcap))) != VJ_OK) return r;
            return D->qB.ensure(sizeof(QEntry) * static_cast<size_t>(qcap));
        }
        char* base = D->arena.as<char>();
        size_t off = 0;
        const size_t cap = D->arena.cap;
        bool fits = true;
        auto carve = [&](DBuf& b, size_t bytes) {
            off = static_cast<size_t>(align_up(static_cast<int64_t>(off), 256));
            bytes = std::max<size_t>(bytes, 256);
            if (off + bytes > cap) {
                fits = false;
                return;
            }
            b.set_view(base + off, bytes);
            off += bytes;
        };
        carve(D->imgs, static_cast<size_t>(imgBytes));
        carve(D->pix, static_cast<size_t>(pixBytes));
        carve(D->iiSum, static_cast<size_t>(iiElems) * 4);
        carve(D->iiSq, static_cast<size_t>(iiElems) * 4);
        carve(D->totS, static_cast<size_t>(totElems) * 4);
        carve(D->totQ, static_cast<size_t>(totElems) * 4);
        carve(D->dets, detBytes);
        if (histTotal) carve(D->ghist, static_cast<size_t>(histTotal) * 4);
        off = static_cast<size_t>(align_up(static_cast<int64_t>(off), 256));
        const int64_t room = fits && off < cap ? static_cast<int64_t>((cap - off) / 2 / sizeof(QEntry)) - 32 : 0;
        const int64_t q = std::min<int64_t>(room, INT32_MAX / 2);
        if (!fits || q < std::max<int64_t>({windowsAll / 8, grpQ, 1}))
            return set_error(VJ_OUT_OF_MEMORY, "detector arena: " + std::to_string(cap) +
                                                   " reserved bytes do not hold this batch");
        qcap = q;
        carve(D->qA, sizeof(QEntry) * static_cast<size_t>(qcap));
        carve(D->qB, sizeof(QEntry) * static_cast<size_t>(qcap));
        return fits ? VJ_OK : set_error(VJ_OUT_OF_MEMORY, "detector arena: queues do not fit");
    };
    int st = layout();
    if (st != VJ_OK) return st;

    std::vector<IIJob32> iij;
    std::vector<CasLevel> lv;
    std::vector<std::vector<ResizeJob>> rj;  // by chain position
    int64_t pixOff = 0, iiOff = 0, tiles = 0, windows = 0, pyrPix = 0;
    const int th = D->cfg.tileRows;
    for (int i = 0; i < nImg; ++i) {
        const uint8_t* base = onDevice ? ims[i].ptr : (mapped[i] ? mapped[i] : D->imgs.as<uint8_t>() + imgOff[i]);
        const int64_t baseStride = onDevice || mapped[i] ? ims[i].stride : imgPitch[i];
        std::vector<const uint8_t*> lp(geo[i].size());
        std::vector<int64_t> ls(geo[i].size());
        for (size_t k = 0; k < geo[i].size(); ++k) {
            const LevelGeom& g = geo[i][k];
            if (g.src == -2) {
                lp[k] = base;
                ls[k] = baseStride;
            } else {
                uint8_t* dst = D->pix.as<uint8_t>() + pixOff;
                const int64_t dstStride = align_up(g.w, 16);
                pixOff += dstStride * g.h;
                ResizeJob r{};
                r.src = g.src >= 0 ? lp[g.src] : base;
                r.srcStride = g.src >= 0 ? ls[g.src] : baseStride;
                r.srcW = g.src >= 0 ? geo[i][g.src].w : ims[i].w;
                r.srcH = g.src >= 0 ? geo[i][g.src].h : ims[i].h;
                r.dst = dst;
                r.dstStride = dstStride;
                r.dstW = g.w;
                r.dstH = g.h;
                r.sx = static_cast<float>(r.srcW) / static_cast<float>(g.w);
                r.sy = static_cast<float>(r.srcH) / static_cast<float>(g.h);
                // chain position: the number of resizes before this one
                int pos = 0;
                for (int q = g.src; q >= 0; q = geo[i][q].src)
                    if (geo[i][q].src != -2) ++pos;
                if (static_cast<int>(rj.size()) <= pos) rj.resize(pos + 1);
                rj[pos].push_back(r);
                lp[k] = dst;
                ls[k] = dstStride;
            }
            IIJob32 J{};
            J.pix = lp[k];
            J.stride = ls[k];
            J.w = g.w;
            J.h = g.h;
            J.pitch = ii_pitch(g.w);
            J.sum = D->iiSum.as<uint32_t>() + iiOff;
            J.sq = D->iiSq.as<uint32_t>() + iiOff;
            iiOff += (g.h + 1) * J.pitch;
            iij.push_back(J);
            CasLevel c{};
            c.sum = J.sum;
            c.sq = J.sq;
            c.pitch = J.pitch;
            c.workW = g.w - D->winW + 1;
            c.workH = g.h - D->winH + 1;
            c.step = g.step;
            c.scanW = (c.workW + g.step - 1) / g.step;
            c.scanH = (c.workH + g.step - 1) / g.step;
            c.tilesX = (c.scanW + 31) / 32;
            c.tileBase = tiles;
            tiles += static_cast<int64_t>(c.tilesX) * ((c.scanH + th - 1) / th);
            windows += static_cast<int64_t>(c.scanW) * c.scanH;
            pyrPix += static_cast<int64_t>(g.w) * g.h;
            c.scale = g.scale;
            c.scaleIdx = g.scaleIdx;
            c.image = i;
            lv.push_back(c);
        }
    }
    const IIPlan ip = plan_integral_jobs(iij.data(), static_cast<int>(iij.size()));

    // ---- plan bytes: [DevPlan][rjFirst][rjItems][ResizeJob...][IIJob...][CasLevel...]
    const int nResize = static_cast<int>(rj.size());
    std::vector<int> rjFirst(nResize + 1, 0);
    std::vector<int64_t> rjItems(std::max(nResize, 1), 0);
    std::vector<ResizeJob> rjAll;
    for (int p = 0; p < nResize; ++p) {
        rjFirst[p] = static_cast<int>(rjAll.size());
        int64_t items = 0;
        for (auto& r : rj[p]) {
            r.itemBase = items;
            items += static_cast<int64_t>(r.dstH) * ((r.dstW + 127) / 128);
            rjAll.push_back(r);
        }
        rjItems[p] = items;
    }
    rjFirst[nResize] = static_cast<int>(rjAll.size());
    const int64_t oFirst = align_up(sizeof(DevPlan), 64);
    const int64_t oItems = align_up(oFirst + sizeof(int) * rjFirst.size(), 64);
    const int64_t oRj = align_up(oItems + sizeof(int64_t) * rjItems.size(), 64);
    const int64_t oII = align_up(oRj + sizeof(ResizeJob) * std::max<size_t>(rjAll.size(), 1), 64);
    const int64_t oLv = align_up(oII + sizeof(IIJob32) * std::max<size_t>(iij.size(), 1), 64);
    const int64_t oHist = align_up(oLv + sizeof(CasLevel) * std::max<size_t>(lv.size(), 1), 64);
    const int64_t planBytes = align_up(oHist + sizeof(int64_t) * histBase.size(), 64);
    if (planBytes > static_cast<int64_t>(D->dplan.cap) || planBytes > static_cast<int64_t>(D->hplan.cap)) {
        const int64_t want = std::max<int64_t>(planBytes, 1 << 20);
        if ((st = D->dplan.ensure(want)) != VJ_OK) return st;
        if ((st = D->hplan.ensure(want)) != VJ_OK) return st;
    }
    if (nImg > D->imageCap) {
        D->imageCap = std::max(nImg, 256);
        if ((st = D->dctrl.ensure(ctrl_bytes(D->imageCap))) != VJ_OK) return st;
        if ((st = D->hctrl.ensure(ctrl_bytes(D->imageCap))) != VJ_OK) return st;
    }
    char* hp = D->hplan.as<char>();
    char* dp = D->dplan.as<char>();
    std::memcpy(hp + oFirst, rjFirst.data(), sizeof(int) * rjFirst.size());
    std::memcpy(hp + oItems, rjItems.data(), sizeof(int64_t) * rjItems.size());
    if (!rjAll.empty()) std::memcpy(hp + oRj, rjAll.data(), sizeof(ResizeJob) * rjAll.size());
    std::memcpy(hp + oII, iij.data(), sizeof(IIJob32) * iij.size());
    std::memcpy(hp + oLv, lv.data(), sizeof(CasLevel) * lv.size());
    std::memcpy(hp + oHist, histBase.data(), sizeof(int64_t) * histBase.size());

    vj_detect_stats& S = D->stats;
    S = vj_detect_stats{};
    S.images = nImg;
    S.levels = static_cast<int64_t>(lv.size());
    S.pyramidPixels = pyrPix;
    S.windows = windows;
    S.queuePasses = static_cast<int>(D->queueEnds.size());

    if (staged) {
        if ((st = D->himgs.ensure(static_cast<size_t>(imgBytes))) != VJ_OK) return st;
        stage_images(ims, imgOff, mapped, D->himgs.as<uint8_t>());
    }

    int64_t hostCap = std::max<int64_t>({int64_t(1) << 16, D->hostHint});
    if (!D->ev0) {
        VJ_CUDA_TRY(cudaEventCreate(&D->ev0));
        VJ_CUDA_TRY(cudaEventCreate(&D->ev1));
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        if (attempt > 0 && (st = layout()) != VJ_OK) return st;
        if ((st = D->hdets.ensure(sizeof(vj_detection) * static_cast<size_t>(hostCap), true)) != VJ_OK) return st;
        DevPlan P{};
        P.nImg = nImg;
        P.nLevels = static_cast<int>(lv.size());
        P.nResize = nResize;
        P.nQueuePasses = static_cast<int>(D->queueEnds.size());
        P.winW = D->winW;
        P.winH = D->winH;
        P.normMode = D->normMode;
        P.nStages = D->nStages;
        P.tileStages = D->tileStages;
        P.deepFrom = D->deepFrom;
        P.qcap = static_cast<int>(qcap);
        P.detCap = detCap;
        for (size_t m = 0; m < D->queueEnds.size(); ++m) P.queueEnd[m] = D->queueEnds[m];
        P.hostCap = static_cast<int>(std::min<int64_t>(hostCap, INT32_MAX));
        P.colWalk = colWalk ? 1 : 0;
        P.spreadStumps = D->spreadStumps ? 1 : 0;
        P.holdBlock = D->testHoldBlock;
        P.barrierTimeoutNs = D->testBarrierTimeoutNs;
        P.totalTiles = tiles;
        P.totS = D->totS.as<uint32_t>();
        P.totQ = D->totQ.as<uint32_t>();
        P.ip = ip;
        P.rjFirst = reinterpret_cast<const int*>(dp + oFirst);
        P.rjItems = reinterpret_cast<const int64_t*>(dp + oItems);
        P.rjobs = reinterpret_cast<const ResizeJob*>(dp + oRj);
        P.iijobs = reinterpret_cast<const IIJob32*>(dp + oII);
        P.levels = reinterpret_cast<const CasLevel*>(dp + oLv);
        P.stumps = D->stumps.as<DStump>();
        P.pstumps.a = D->pstumps.as<uint4>();
        P.pstumps.b = P.pstumps.a + D->nStumps;
        P.pstumps.c = P.pstumps.b + D->nStumps;
        P.stages = D->stages.as<DStage>();
        P.q[0] = D->qA.as<QEntry>();
        P.q[1] = D->qB.as<QEntry>();
        P.dets = D->dets.as<vj_detection>();
        P.ctrl = D->dctrl.as<CtrlHead>();
        P.counts = reinterpret_cast<int*>(D->dctrl.as<char>() + align_up(sizeof(CtrlHead), 16));
        P.offsets = P.counts + D->imageCap;
        P.rawOff = P.offsets + D->imageCap;
        P.ccount = P.rawOff + D->imageCap;
        P.gcount = P.ccount + D->imageCap;
        P.selKey = reinterpret_cast<unsigned long long*>(D->dctrl.as<char>() + ctrl_sel_offset(D->imageCap));
        P.hostDets = static_cast<vj_detection*>(D->hdets.dev);
        if (ga.on) {
            GroupPlan& g = P.grp;
            g.enabled = 1;
            g.minN = std::max(1, ga.minN);
            g.limit = std::max(1, ga.limit);
            g.cap = static_cast<int>(group_slots(D->qA.cap, D->qB.cap));
            g.eps = 0.2f;
            g.histBase = reinterpret_cast<const int64_t*>(dp + oHist);
            g.hist = D->ghist.as<int>();
            g.histTotal = histTotal;
            carve_group(g, D->qA.as<char>(), D->qB.as<char>(), g.cap);
        }
        std::memcpy(hp, &P, sizeof(P));
        if ((st = ensure_graph(D, static_cast<size_t>(planBytes))) != VJ_OK) return st;
        if (D->graphPlanBytes != static_cast<size_t>(planBytes)) {
            VJ_CUDA_TRY(cudaGraphExecMemcpyNodeSetParams1D(D->exec, D->planNode, D->dplan.p, D->hplan.p,
                                                           static_cast<size_t>(planBytes), cudaMemcpyHostToDevice));
            D->graphPlanBytes = static_cast<size_t>(planBytes);
        }
        if (staged) {
            VJ_CUDA_TRY(cudaMemcpyAsync(D->imgs.p, D->himgs.p, static_cast<size_t>(imgBytes), cudaMemcpyHostToDevice, s));
        } else if (!onDevice) {
            for (int i = 0; i < nImg; ++i) {
                if (ims[i].h <= 0 || ims[i].w <= 0 || mapped[i]) continue;
                uint8_t* d = D->imgs.as<uint8_t>() + imgOff[i];
                if (dense[i])
                    VJ_CUDA_TRY(cudaMemcpyAsync(d, ims[i].ptr, static_cast<size_t>(imgPitch[i] * (ims[i].h - 1) + ims[i].w),
                                                cudaMemcpyHostToDevice, s));
                else
                    VJ_CUDA_TRY(cudaMemcpy2DAsync(d, imgPitch[i], ims[i].ptr, ims[i].stride, ims[i].w, ims[i].h,
                                                  cudaMemcpyHostToDevice, s));
            }
        }
        {
            std::unique_lock<std::mutex> chainLock;
            if (D->chain) {
                chainLock = std::unique_lock<std::mutex>(D->chain->mu);
                if (D->chain->last) VJ_CUDA_TRY(cudaStreamWaitEvent(s, D->chain->last, 0));
            }
            VJ_CUDA_TRY(cudaEventRecord(D->ev0, s));
            cudaError_t le = cudaSuccess;
            VJ_TIMED_LAUNCH("detect_persistent_kernel", s, le = cudaGraphLaunch(D->exec, s));
            if (le != cudaSuccess)
                return set_error(VJ_CUDA_ERROR, std::string("detection graph launch: ") + cudaGetErrorString(le));
            VJ_CUDA_TRY(cudaEventRecord(D->ev1, s));
            if (D->chain) {
                if (!D->chain->last) VJ_CUDA_TRY(cudaEventCreateWithFlags(&D->chain->last, cudaEventDisableTiming));
                VJ_CUDA_TRY(cudaEventRecord(D->chain->last, s));
            }
        }
        const double t1 = now_ms();
        VJ_CUDA_TRY(cudaStreamSynchronize(s));
        const double t2 = now_ms();
        float ms = 0.0f;
        VJ_CUDA_TRY(cudaEventElapsedTime(&ms, D->ev0, D->ev1));
        const CtrlHead* H = D->hctrl.as<CtrlHead>();
        if (H->sync.error) return set_error(VJ_RUNTIME_ERROR, "detection kernel: a grid barrier wait timed out");
        if (ga.on && H->grpError) return set_error(VJ_RUNTIME_ERROR, "detection kernel: grouping stopped on an error");
        const int* hc = reinterpret_cast<const int*>(D->hctrl.as<char>() + align_up(sizeof(CtrlHead), 16));
        int need = 0, qneed = 0;
        int64_t total = 0;
        for (int i = 0; i < nImg; ++i) {
            need = std::max(need, hc[i]);
            total += hc[i];
        }
        for (int k = 0; k < kQueues; ++k) qneed = std::max(qneed, H->qcount[k]);
        D->qHint = std::max<int64_t>(D->qHint, qneed + qneed / 4);
        D->detHint = std::max(D->detHint, need + need / 4);
        D->hostHint = std::max<int64_t>(D->hostHint, total + total / 4);
        S.attempts = attempt + 1;
        if (ga.on) D->grpHint = std::max<int64_t>(D->grpHint, H->compactTotal + H->compactTotal / 4);
        if (qneed > qcap || need > detCap || H->compactOverflow || (ga.on && H->grpOverflow)) {
            const int64_t gq = ga.on ? (D->grpHint * kGroupBytesB + 16 * 256) / static_cast<int64_t>(sizeof(QEntry)) + 1 : 0;
            qcap = std::min<int64_t>(std::max<int64_t>({qcap, qneed + qneed / 4, gq}), INT32_MAX / 2);
            detCap = std::max(detCap, need + need / 4);
            hostCap = std::max<int64_t>(hostCap, total + total / 4);
            continue;
        }
        S.gpuMs = ms;
        S.hostMs[0] = t1 - t0;
        S.hostMs[1] = t2 - t1;
        S.gated = static_cast<int64_t>(H->stats[0]);
        S.stumpEvals = static_cast<int64_t>(H->stats[1]);
        S.rawDetections = H->compactTotal;
        S.deepWindows = D->deepFrom < D->nStages ? H->qcount[D->queueEnds.size()] : 0;
        for (int k = 0; k < kPhaseStamps - 1; ++k) {
            const unsigned long long a = H->sync.stamp[k], b = H->sync.stamp[k + 1];
            S.phaseMs[k] = (a && b >= a) ? static_cast<double>(b - a) * 1e-6 : 0.0;
        }
        *outCounts = hc;
        *outOffsets = hc + D->imageCap;
        *outDetCap = detCap;
        if (outGrouped) *outGrouped = hc + 4 * D->imageCap;
        return VJ_OK;
    }
    return set_error(VJ_RUNTIME_ERROR, "detection buffers still overflow after growing them");
}

int run_batch(vj_detector* D, const std::vector<BatchImage>& ims, bool onDevice, float sf, int minN, int minObj,
              int maxDet, bool group, vj_detection* out, int capPer, int* counts, cudaStream_t s) {
    const int* hc = nullptr;
    const int* ho = nullptr;
    const int* hg = nullptr;
    int detCap = 0;
    GroupArgs ga;
    ga.on = group;
    ga.minN = minN;
    ga.limit = std::max(1, maxDet);
    const int st = execute(D, ims, onDevice, sf, minObj, ga, s, &hc, &ho, &detCap, &hg);
    if (st != VJ_OK) return st;
    const double t0 = now_ms();
    const int nImg = static_cast<int>(ims.size());
    if (group) {
        // grouped on the device: copy each image's clusters out
        const vj_detection* hd = D->hdets.as<vj_detection>();
        for (int i = 0; i < nImg; ++i) {
            const int k = std::min(hg[i], capPer);
            if (k > 0) std::memcpy(out + static_cast<size_t>(i) * capPer, hd + ho[i], sizeof(vj_detection) * k);
            counts[i] = k;
        }
        D->stats.hostMs[2] = now_ms() - t0;
        return VJ_OK;
    }
    const int limit = std::max(1, maxDet);
    const vj_detection* hd = D->hdets.as<vj_detection>();
    // raw detections: canonical order, the first maxDet of each image
    auto post = [&](int i) {
        const vj_detection* src = hd + ho[i];
        std::vector<vj_detection> raw(src, src + std::min(hc[i], detCap));
        canonical_sort(raw);
        if (static_cast<int>(raw.size()) > limit) raw.resize(limit);
        const int k = std::min(static_cast<int>(raw.size()), capPer);
        if (k > 0) std::memcpy(out + static_cast<size_t>(i) * capPer, raw.data(), sizeof(vj_detection) * k);
        counts[i] = k;
    };
    if (nImg >= 8) {
        const int T = std::min(16, std::max(1, static_cast<int>(std::thread::hardware_concurrency())));
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                for (int i = t; i < nImg; i += T) post(i);
            });
        for (auto& x : th) x.join();
    } else {
        for (int i = 0; i < nImg; ++i) post(i);
    }
    D->stats.hostMs[2] = now_ms() - t0;
    return VJ_OK;
}

int check_config(const vj_detect_config& c) {
    if ((c.tileRows != 4 && c.tileRows != 8 && c.tileRows != 16) || c.tileStumps < 0 || c.queueStumps < 0 ||
        c.blocksPerSM < 0 || (c.deepSlots != 1 && c.deepSlots != 2) || c.reserved != 0)
        return set_error(VJ_INVALID_ARG,
                         "detection config: tileRows must be 4, 8 or 16, deepSlots 1 or 2, the rest >= 0");
    return VJ_OK;
}

int collect_images(vj_detector* d, int n, const uint8_t* const* images, const int* w, const int* h,
                   const int* stride, const char* fn, std::vector<BatchImage>* ims) {
    ims->resize(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        if (!images[i] || w[i] <= 0 || h[i] <= 0 || stride[i] < w[i] || w[i] > d->maxW || h[i] > d->maxH)
            return set_error(VJ_INVALID_ARG, std::string(fn) + ": bad image " + std::to_string(i));
        (*ims)[static_cast<size_t>(i)] = BatchImage{images[i], w[i], h[i], stride[i]};
    }
    return VJ_OK;
}

}  // namespace

namespace vjgb {

int detector_set_launch_chain(vj_detector* d, LaunchChain* chain) {
    if (!d) return set_error(VJ_INVALID_ARG, "detector_set_launch_chain: null detector");
    d->chain = chain;
    return ok();
}

}  // namespace vjgb

extern "C" {

int vj_detector_create(int winW, int winH, int maxImageW, int maxImageH, int maxDetections, vj_detector** out) {
    if (!out) return set_error(VJ_INVALID_ARG, "vj_detector_create: null out");
    *out = nullptr;
    if (winW < 3 || winH < 3 || winW > 64 || winH > 64 || maxImageW <= 0 || maxImageH <= 0 || maxDetections <= 0 ||
        maxImageW > 65535 || maxImageH > 65535)
        return set_error(VJ_INVALID_ARG, "vj_detector_create: invalid constructor args");
    auto* d = new vj_detector();
    d->winW = winW;
    d->winH = winH;
    d->maxW = maxImageW;
    d->maxH = maxImageH;
    d->maxDet = maxDetections;
    *out = d;
    return ok();
}

int vj_detector_destroy(vj_detector* d) {
    if (!d) return ok();
    drop_graph(d);
    if (d->ev0) cudaEventDestroy(d->ev0);
    if (d->ev1) cudaEventDestroy(d->ev1);
    for (DBuf* b : {&d->stumps, &d->pstumps, &d->stages, &d->imgs, &d->pix, &d->iiSum, &d->iiSq, &d->totS, &d->totQ,
                    &d->qA, &d->qB, &d->dets, &d->dplan, &d->dctrl, &d->ghist, &d->arena})
        b->release();
    d->hplan.release();
    d->hctrl.release();
    d->hdets.release();
    d->himgs.release();
    delete d;
    return ok();
}

int vj_detector_clear_model(vj_detector* d) {
    if (!d) return set_error(VJ_INVALID_ARG, "vj_detector_clear_model: null detector");
    d->stumps.release();
    d->pstumps.release();
    d->stages.release();
    d->nStages = d->nStumps = 0;
    d->hStages.clear();
    return ok();
}

// Reorders each stage's deep-pass records within blocks of kDeepBlock stumps
// so that the stumps one deep-pass load instruction reads spread over the
// shared-memory banks.  Lane j of a slot evaluates stump k0 + 16 ev + j (k0 a
// multiple of kDeepBlock from the stage's first stump), and the two slots'
// patches are interleaved (element o of slot s at 2 o + s), so a slot's load
// of corner c touches bank 2 (o mod 16) + s: one wavefront when the 16 stumps
// of a group that load corner c have distinct o mod 16.  A seeded local
// search swaps stumps between the groups of a block while the sum, over
// groups and corners, of the largest bank count does not grow.  A record
// keeps its position in the block before the reordering in bits 10-15 of its
// first offset's half-word (offsets stay below 1024); the deep pass's exact
// replay adds the values in that order.  Returns false, leaving the order,
// when the patch has 1,024 elements or more or two stages' stump ranges
// overlap.
struct DeepCorners {
    uint16_t off[12];
    bool three;  // the third rectangle is evaluated (three rectangles, w2 != 0)
};

static bool spread_banks(std::vector<uint4>& pa, std::vector<uint4>& pb, std::vector<uint4>& pc,
                         const std::vector<DeepCorners>& dc, const vj_cascade_stage* stages, int64_t stageCount,
                         int patchElems) {
    const int64_t n = static_cast<int64_t>(pa.size());
    if (patchElems > 1024) return false;
    std::vector<char> seen(static_cast<size_t>(n), 0);
    for (int64_t i = 0; i < stageCount; ++i)
        for (int64_t k = stages[i].first; k < static_cast<int64_t>(stages[i].first) + stages[i].ntrees; ++k) {
            if (seen[static_cast<size_t>(k)]) return false;
            seen[static_cast<size_t>(k)] = 1;
        }
    // the corners the deep pass reads (patch_stump_value: a corner equal to
    // an earlier one is not read again)
    auto loads = [&](int64_t r, int c) {
        const uint16_t* o = dc[static_cast<size_t>(r)].off;
        if (c < 4) return true;
        if (c < 8) return o[c] != o[c - 4];
        if (!dc[static_cast<size_t>(r)].three) return false;
        if (c == 8) return o[8] != o[7];
        if (c == 11) return o[11] != o[3];
        return true;
    };
    uint64_t rng = 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        rng ^= rng << 13;
        rng ^= rng >> 7;
        rng ^= rng << 17;
        return rng;
    };
    for (int64_t si = 0; si < stageCount; ++si) {
        const int64_t first = stages[si].first, nt = stages[si].ntrees;
        for (int64_t b0 = 0; b0 < nt; b0 += kDeepBlock) {
            const int len = static_cast<int>(std::min<int64_t>(kDeepBlock, nt - b0));
            const int ng = (len + 15) / 16;
            std::vector<int> pos(static_cast<size_t>(len));  // block position -> stump (index in the block)
            for (int t = 0; t < len; ++t) pos[t] = t;
            if (ng > 1) {
                // cnt[(g * 12 + c) * 16 + bank]
                std::vector<int> cnt(static_cast<size_t>(ng) * 12 * 16, 0);
                auto add = [&](int g, int r, int dlt) {
                    for (int c = 0; c < 12; ++c)
                        if (loads(first + b0 + r, c))
                            cnt[(static_cast<size_t>(g) * 12 + c) * 16 + (dc[static_cast<size_t>(first + b0 + r)].off[c] & 15)] += dlt;
                };
                auto cost = [&](int g) {
                    int sum = 0;
                    for (int c = 0; c < 12; ++c) {
                        const int* q = &cnt[(static_cast<size_t>(g) * 12 + c) * 16];
                        int m = 0;
                        for (int bk = 0; bk < 16; ++bk) m = std::max(m, q[bk]);
                        sum += m;
                    }
                    return sum;
                };
                for (int t = 0; t < len; ++t) add(t / 16, pos[t], 1);
                std::vector<int> gc(static_cast<size_t>(ng));
                for (int g = 0; g < ng; ++g) gc[g] = cost(g);
                for (int it = 0; it < 1500; ++it) {
                    const int x = static_cast<int>(next() % static_cast<uint64_t>(len));
                    const int y = static_cast<int>(next() % static_cast<uint64_t>(len));
                    const int gx = x / 16, gy = y / 16;
                    if (gx == gy) continue;
                    add(gx, pos[x], -1), add(gy, pos[y], -1), add(gx, pos[y], 1), add(gy, pos[x], 1);
                    const int cx = cost(gx), cy = cost(gy);
                    if (cx + cy <= gc[gx] + gc[gy]) {
                        std::swap(pos[x], pos[y]);
                        gc[gx] = cx, gc[gy] = cy;
                    } else {
                        add(gx, pos[y], -1), add(gy, pos[x], -1), add(gx, pos[x], 1), add(gy, pos[y], 1);
                    }
                }
            }
            std::vector<uint4> ra(pa.begin() + first + b0, pa.begin() + first + b0 + len);
            std::vector<uint4> rb(pb.begin() + first + b0, pb.begin() + first + b0 + len);
            std::vector<uint4> rc(pc.begin() + first + b0, pc.begin() + first + b0 + len);
            for (int t = 0; t < len; ++t) {
                const size_t at = static_cast<size_t>(first + b0 + t), from = static_cast<size_t>(pos[t]);
                pa[at] = ra[from];
                pb[at] = rb[from];
                pc[at] = rc[from];
                pb[at].z |= static_cast<uint32_t>(pos[t]) << 10;
            }
        }
    }
    return true;
}

int vj_detector_set_model(vj_detector* d, const vj_haar_feature* features, int64_t featureCount,
                          const vj_stump4* stumps, int64_t stumpCount, const vj_cascade_stage* stages,
                          int64_t stageCount) {
    if (!d || !features || !stumps || !stages || featureCount <= 0 || stumpCount <= 0 || stageCount <= 0 ||
        stumpCount > INT32_MAX || stageCount > INT32_MAX)
        return set_error(VJ_INVALID_ARG, "vj_detector_set_model: bad arguments");
    const int mW = d->winW + 1;
    const int patchElems = (d->winW + 1) * (d->winH + 1);
    std::vector<DStump> ds(static_cast<size_t>(stumpCount));
    std::vector<uint4> pa(static_cast<size_t>(stumpCount)), pb(pa.size()), pc(pa.size());
    std::vector<DeepCorners> dc(pa.size());
    for (int64_t i = 0; i < stumpCount; ++i) {
        const int32_t fi = float_bits(stumps[i].featureBits);
        if (fi < 0 || fi >= featureCount)
            return set_error(VJ_INVALID_ARG, "vj_detector_set_model: stump references a missing feature");
        const vj_haar_feature& f = features[fi];
        DStump& o = ds[static_cast<size_t>(i)];
        std::memset(&o, 0, sizeof(o));
        o.theta = stumps[i].theta;
        o.left = stumps[i].leftVal;
        o.right = stumps[i].rightVal;
        o.nr = f.rectCount == 3 ? 3 : 2;
        const vj_fast_rect* rr[3] = {&f.r0, &f.r1, &f.r2};
        uint16_t off[12] = {0};
        for (int r = 0; r < 3; ++r) {
            o.w[r] = rr[r]->w;
            const int32_t p[4] = {rr[r]->p0, rr[r]->p1, rr[r]->p2, rr[r]->p3};
            for (int c = 0; c < 4; ++c) {
                // BuildFeatureLUTKernel's decode (face_vision_engine.cu:360-365).
                const int dy = p[c] / mW, dx = p[c] - dy * mW;
                if (r < o.nr && (dx < 0 || dx > d->winW || dy < 0 || dy > d->winH || p[c] >= patchElems))
                    return set_error(VJ_INVALID_ARG, "vj_detector_set_model: feature corner outside the window");
                o.dx[4 * r + c] = static_cast<int8_t>(r < o.nr ? dx : 0);
                o.dy[4 * r + c] = static_cast<int8_t>(r < o.nr ? dy : 0);
                off[4 * r + c] = static_cast<uint16_t>(r < o.nr ? p[c] : 0);
            }
        }
        uint32_t ow[6];
        for (int k = 0; k < 6; ++k)
            ow[k] = static_cast<uint32_t>(off[2 * k]) | (static_cast<uint32_t>(off[2 * k + 1]) << 16);
        const size_t j = static_cast<size_t>(i);
        pa[j] = make_uint4(static_cast<uint32_t>(float_bits(o.theta)), static_cast<uint32_t>(float_bits(o.left)),
                           static_cast<uint32_t>(float_bits(o.right)), static_cast<uint32_t>(float_bits(rr[0]->w)));
        pb[j] = make_uint4(static_cast<uint32_t>(float_bits(rr[1]->w)),
                           static_cast<uint32_t>(float_bits(o.nr == 3 ? rr[2]->w : 0.0f)), ow[0], ow[1]);
        pc[j] = make_uint4(ow[2], ow[3], ow[4], ow[5]);
        std::memcpy(dc[j].off, off, sizeof(off));
        dc[j].three = o.nr == 3 && rr[2]->w != 0.0f;
    }
    std::vector<DStage> dst(static_cast<size_t>(stageCount));
    for (int64_t i = 0; i < stageCount; ++i) {
        if (stages[i].ntrees < 0 || stages[i].first < 0 ||
            static_cast<int64_t>(stages[i].first) + stages[i].ntrees > stumpCount)
            return set_error(VJ_INVALID_ARG, "vj_detector_set_model: stage outside the stump array");
        // tolerance of the deep pass's order-free stage sums (cascade.cuh deep_pass)
        double lim = 0.0;
        for (int k = 0; k < stages[i].ntrees; ++k) {
            const vj_stump4& sk = stumps[stages[i].first + k];
            lim += std::max(std::fabs(static_cast<double>(sk.leftVal)), std::fabs(static_cast<double>(sk.rightVal)));
        }
        const double u = std::ldexp(1.0, -24), nt = stages[i].ntrees;
        auto gamma = [&](double k) { return k * u / (1.0 - k * u); };
        // relative rounding of both sums, plus half an ulp of the smallest
        // subnormal per operation, rounded up to a float
        const double bound = 1.01 * (gamma(nt - 1.0 > 0.0 ? nt - 1.0 : 0.0) + gamma(nt + 5.0)) * lim +
                             (2.0 * nt + 6.0) * std::ldexp(1.0, -150);
        const float tol = std::nextafter(static_cast<float>(bound), INFINITY);
        dst[static_cast<size_t>(i)] = DStage{stages[i].first, stages[i].ntrees, stages[i].threshold, tol};
    }
    int st;
    if ((st = d->stumps.ensure(sizeof(DStump) * ds.size())) != VJ_OK) return st;
    if ((st = d->pstumps.ensure(sizeof(uint4) * 3 * pa.size())) != VJ_OK) return st;
    if ((st = d->stages.ensure(sizeof(DStage) * dst.size())) != VJ_OK) return st;
    VJ_CUDA_TRY(cudaMemcpy(d->stumps.p, ds.data(), sizeof(DStump) * ds.size(), cudaMemcpyHostToDevice));
    const bool spread = spread_banks(pa, pb, pc, dc, stages, stageCount, patchElems);
    for (int k = 0; k < 3; ++k) {
        const std::vector<uint4>& plane = k == 0 ? pa : (k == 1 ? pb : pc);
        VJ_CUDA_TRY(cudaMemcpy(d->pstumps.as<uint4>() + k * pa.size(), plane.data(), sizeof(uint4) * plane.size(),
                               cudaMemcpyHostToDevice));
    }
    VJ_CUDA_TRY(cudaMemcpy(d->stages.p, dst.data(), sizeof(DStage) * dst.size(), cudaMemcpyHostToDevice));
    d->nStages = static_cast<int>(stageCount);
    d->nStumps = static_cast<int>(stumpCount);
    d->spreadStumps = spread;
    d->hStages = dst;
    schedule_passes(d);
    return ok();
}

int vj_detector_set_norm_mode(vj_detector* d, int mode) {
    if (!d || (mode != VJ_NORM_FLOAT_CORNERS && mode != VJ_NORM_EXACT_INT))
        return set_error(VJ_INVALID_ARG, "vj_detector_set_norm_mode: bad arguments");
    d->normMode = mode;
    return ok();
}

int vj_detector_set_config(vj_detector* d, const vj_detect_config* cfg) {
    if (!d || !cfg) return set_error(VJ_INVALID_ARG, "vj_detector_set_config: null argument");
    const int st = check_config(*cfg);
    if (st != VJ_OK) return st;
    d->cfg = *cfg;
    if (d->nStages > 0) schedule_passes(d);
    return ok();
}

int vj_detector_get_config(const vj_detector* d, vj_detect_config* cfg) {
    if (!d || !cfg) return set_error(VJ_INVALID_ARG, "vj_detector_get_config: null argument");
    *cfg = d->cfg;
    return ok();
}

int vj_detector_reserve(vj_detector* d, int64_t bytes) {
    if (!d || bytes < 0) return set_error(VJ_INVALID_ARG, "vj_detector_reserve: bad arguments");
    for (DBuf* b : {&d->imgs, &d->pix, &d->iiSum, &d->iiSq, &d->totS, &d->totQ, &d->qA, &d->qB, &d->dets, &d->ghist})
        b->release();
    d->arena.release();
    if (bytes == 0) return ok();
    const cudaError_t e = cudaMalloc(&d->arena.p, static_cast<size_t>(bytes));
    if (e != cudaSuccess) {
        d->arena.p = nullptr;
        return set_error(VJ_OUT_OF_MEMORY, std::string("vj_detector_reserve: ") + cudaGetErrorString(e));
    }
    d->arena.cap = static_cast<size_t>(bytes);
    return ok();
}

int vj_detector_occupancy(vj_detector* d, int* blocksPerSM) {
    if (!d || !blocksPerSM) return set_error(VJ_INVALID_ARG, "vj_detector_occupancy: null argument");
    const int th = d->cfg.tileRows;
    const size_t smem = smem_bytes(d, th);
    const void* fn = kernel_ptr(d->cfg);
    VJ_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int fit = 0;
    VJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, kCasThreads, smem));
    *blocksPerSM = fit;
    return ok();
}

int vj_detector_device_bytes(const vj_detector* d, int64_t* bytes) {
    if (!d || !bytes) return set_error(VJ_INVALID_ARG, "vj_detector_device_bytes: null argument");
    int64_t t = 0;
    for (const DBuf* b : {&d->stumps, &d->pstumps, &d->stages, &d->imgs, &d->pix, &d->iiSum, &d->iiSq,
                          &d->totS, &d->totQ, &d->qA, &d->qB, &d->dets, &d->dplan, &d->dctrl, &d->ghist, &d->arena})
        if (!b->view) t += static_cast<int64_t>(b->cap);
    *bytes = t;
    return ok();
}

int vj_detect_estimate_bytes(int winW, int winH, int w, int h, float scaleFactor, int minObjectSize,
                             int maxDetections, int64_t* bytes) {
    if (!bytes || winW < 3 || winH < 3 || w <= 0 || h <= 0 || !(scaleFactor > 1.0f) || minObjectSize < 1)
        return set_error(VJ_INVALID_ARG, "vj_detect_estimate_bytes: bad arguments");
    int64_t t = align_up(w, 16) * h + 4 * (static_cast<int64_t>(w) + 1);  // image copy, grouping histogram
    for (const LevelGeom& g : plan_levels(w, h, winW, winH, scaleFactor, minObjectSize)) {
        if (g.src != -2) t += align_up(g.w, 16) * g.h;           // resized level
        const int64_t ii = static_cast<int64_t>(g.h + 1) * ii_pitch(g.w);
        t += ii * 8;                                               // sums + squared sums (32-bit)
        t += static_cast<int64_t>(col_segs(g.h)) * col_chunks(g.w) * 32 * 8;  // segment totals
        const int64_t win = static_cast<int64_t>((g.w - winW + g.step) / g.step) * ((g.h - winH + g.step) / g.step);
        t += 2 * static_cast<int64_t>(sizeof(QEntry)) * (win / 8 + 1);        // two queues
        t += static_cast<int64_t>(sizeof(CasLevel) + sizeof(IIJob32) + sizeof(ResizeJob));
    }
    t += static_cast<int64_t>(sizeof(vj_detection)) * std::max(64, std::min(std::max(1, maxDetections), 4096));
    *bytes = t + t / 8;  // the work buffers grow with an eighth of slack
    return ok();
}

int vj_detect(vj_detector* d, const uint8_t* image, int w, int h, int stride, int image_on_device, float scaleFactor,
              int minNeighbors, int minObjectSize, int maxDetections, int applyGrouping, vj_detection* out,
              int capacity, int* count, void* stream) {
    if (count) *count = 0;
    if (!d || !image || !out || !count || w <= 0 || h <= 0 || stride < w || !(scaleFactor > 1.0f) ||
        minObjectSize < 1 || capacity < 0)
        return set_error(VJ_INVALID_ARG, "vj_detect: bad arguments");
    if (d->nStages <= 0) return set_error(VJ_INVALID_ARG, "vj_detect: no cascade model set");
    if (w > d->maxW || h > d->maxH) return set_error(VJ_INVALID_ARG, "vj_detect: image larger than the detector");
    const int maxDet = std::max(1, std::min(maxDetections, d->maxDet));
    std::vector<BatchImage> ims{{image, w, h, stride}};
    const int st = run_batch(d, ims, image_on_device != 0, scaleFactor, minNeighbors, minObjectSize, maxDet,
                             applyGrouping != 0, out, capacity, count, static_cast<cudaStream_t>(stream));
    return st == VJ_OK ? ok() : st;
}

int vj_group_rectangles(const vj_detection* in, int n, int minNeighbors, float eps, vj_detection* out, int* count) {
    if (!count || n < 0 || (n > 0 && (!in || !out))) return set_error(VJ_INVALID_ARG, "vj_group_rectangles: bad arguments");
    const std::vector<vj_detection> v(in, in + n);
    const std::vector<vj_detection> g = group_rectangles(v, minNeighbors, eps);
    if (!g.empty()) std::memcpy(out, g.data(), sizeof(vj_detection) * g.size());
    *count = static_cast<int>(g.size());
    return ok();
}

int vj_detect_batch(vj_detector* d, int n, const uint8_t* const* images, const int* w, const int* h,
                    const int* stride, int images_on_device, float scaleFactor, int minNeighbors, int minObjectSize,
                    int maxDetectionsPerImage, int applyGrouping, vj_detection* out, int capPerImage, int* counts,
                    void* stream) {
    if (!d || n <= 0 || !images || !w || !h || !stride || !out || !counts || !(scaleFactor > 1.0f) ||
        minObjectSize < 1 || capPerImage < 0)
        return set_error(VJ_INVALID_ARG, "vj_detect_batch: bad arguments");
    if (d->nStages <= 0) return set_error(VJ_INVALID_ARG, "vj_detect_batch: no cascade model set");
    std::vector<BatchImage> ims;
    int st = collect_images(d, n, images, w, h, stride, "vj_detect_batch", &ims);
    if (st != VJ_OK) return st;
    for (int i = 0; i < n; ++i) counts[i] = 0;
    const int maxDet = std::max(1, std::min(maxDetectionsPerImage, d->maxDet));
    st = run_batch(d, ims, images_on_device != 0, scaleFactor, minNeighbors, minObjectSize, maxDet,
                   applyGrouping != 0, out, capPerImage, counts, static_cast<cudaStream_t>(stream));
    return st == VJ_OK ? ok() : st;
}

int vj_detector_test_barrier_timeout(vj_detector* d, int holdBlock, int64_t timeoutNs) {
    if (!d || holdBlock < -1 || timeoutNs < 0)
        return set_error(VJ_INVALID_ARG, "vj_detector_test_barrier_timeout: bad arguments");
    d->testHoldBlock = holdBlock;
    d->testBarrierTimeoutNs = static_cast<unsigned long long>(timeoutNs);
    return ok();
}

int vj_detector_last_stats(const vj_detector* d, vj_detect_stats* out) {
    if (!d || !out) return set_error(VJ_INVALID_ARG, "vj_detector_last_stats: null argument");
    *out = d->stats;
    return ok();
}

int vj_detector_autotune(vj_detector* d, int n, const uint8_t* const* images, const int* w, const int* h,
                         const int* stride, int images_on_device, float scaleFactor, int minObjectSize, int repeats,
                         vj_detect_config* chosen, double* chosenMs) {
    if (!d || n <= 0 || !images || !w || !h || !stride || !(scaleFactor > 1.0f) || minObjectSize < 1)
        return set_error(VJ_INVALID_ARG, "vj_detector_autotune: bad arguments");
    if (d->nStages <= 0) return set_error(VJ_INVALID_ARG, "vj_detector_autotune: no cascade model set");
    std::vector<BatchImage> ims;
    int st = collect_images(d, n, images, w, h, stride, "vj_detector_autotune", &ims);
    if (st != VJ_OK) return st;
    repeats = std::max(1, repeats);
    // Candidate tile-pass depths: the cumulative stump counts at the ends of
    // the first stages (the tile pass covers whole stages).
    std::vector<int> depths;
    int acc = 0;
    for (int s = 0; s < d->nStages && s < 7; ++s) {
        acc += d->hStages[s].ntrees;
        depths.push_back(acc);
    }
    // Two rounds: first the tile shape and residency at the current tile-pass
    // depth, then the depth with the best of those.  Every candidate's raw
    // detections must equal the first candidate's.
    const vj_detect_config saved = d->cfg;
    std::vector<std::vector<vj_detection>> ref;
    double bestMs = 0.0;
    vj_detect_config bestCfg = saved;
    bool have = false;
    auto trial = [&](const vj_detect_config& cand) -> int {
        d->cfg = cand;
        schedule_passes(d);
        const int* hc = nullptr;
        const int* ho = nullptr;
        int detCap = 0;
        int r = execute(d, ims, images_on_device != 0, scaleFactor, minObjectSize, GroupArgs{}, nullptr, &hc, &ho,
                        &detCap);
        if (r != VJ_OK) return r;
        std::vector<std::vector<vj_detection>> got(static_cast<size_t>(n));
        const vj_detection* hd = d->hdets.as<vj_detection>();
        for (int i = 0; i < n; ++i) {
            got[i].assign(hd + ho[i], hd + ho[i] + std::min(hc[i], detCap));
            std::sort(got[i].begin(), got[i].end(), canonical_less);
        }
        if (ref.empty()) {
            ref = std::move(got);
        } else {
            for (int i = 0; i < n; ++i)
                if (got[i].size() != ref[i].size() ||
                    (!got[i].empty() &&
                     std::memcmp(got[i].data(), ref[i].data(), sizeof(vj_detection) * got[i].size()) != 0))
                    return set_error(VJ_RUNTIME_ERROR,
                                     "vj_detector_autotune: configurations disagree on image " + std::to_string(i));
        }
        std::vector<double> t;
        for (int k = 0; k < repeats; ++k) {
            r = execute(d, ims, images_on_device != 0, scaleFactor, minObjectSize, GroupArgs{}, nullptr, &hc, &ho,
                        &detCap);
            if (r != VJ_OK) return r;
            t.push_back(d->stats.gpuMs);
        }
        std::sort(t.begin(), t.end());
        const double med = t[t.size() / 2];
        if (!have || med < bestMs) {
            have = true;
            bestMs = med;
            bestCfg = cand;
        }
        return VJ_OK;
    };
    for (int th : {8, 4, 16})
        for (int bps : {4, 0})
            for (int slots : {2, 1}) {
                if (st != VJ_OK) break;
                vj_detect_config c = saved;
                c.tileRows = th;
                c.blocksPerSM = bps;
                c.deepSlots = slots;
                c.queueStumps = 0;
                st = trial(c);
            }
    const vj_detect_config shape = bestCfg;
    for (int dep : depths) {
        if (st != VJ_OK) break;
        vj_detect_config c = shape;
        c.tileStumps = dep;
        st = trial(c);
    }
    const int best = have ? 0 : -1;
    if (st != VJ_OK || best < 0) {
        d->cfg = saved;
        schedule_passes(d);
        return st != VJ_OK ? st : set_error(VJ_RUNTIME_ERROR, "vj_detector_autotune: no candidate ran");
    }
    d->cfg = bestCfg;
    schedule_passes(d);
    if (chosen) *chosen = d->cfg;
    if (chosenMs) *chosenMs = bestMs;
    return ok();
}

}  // extern "C"
