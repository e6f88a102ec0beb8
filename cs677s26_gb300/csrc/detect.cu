// Multiscale cascade detection on sm_103a, for one image (vj_detect, the
// drop-in for FaceVisionEngine::detectMultiScale, src/face_vision_engine.cu:
// 1541-1747) or many images at once (vj_detect_batch).
//
// Per call:
//   1. pyramid: level k is resized from the previous scanned level with the
//      reference's pixel-centre bilinear arithmetic (face_vision_engine.cu:
//      270-308, main.cu:545-585); one launch per chain position covers that
//      level of every image;
//   2. integral images of every level of every image: one launch per pass
//      (integral.cu);
//   3. tile pass: each warp takes a 32x8 block of windows of some level
//      (dynamic work counter over all levels of all images), applies the
//      variance gate (face_vision_engine.cu:484-492), runs the first cascade
//      stages and compacts the surviving windows with warp ballots between
//      stages;
//   4. queue passes: the survivors of the early stages from all tiles are
//      taken 256 at a time per warp and run through the next group of
//      stages the same way, so deep stages also run on full warps;
//   5. the survivors of the last stage become Detection records; the host
//      sorts them into the reference CPU path's order (level, y, x),
//      truncates to maxDetections and groups them (groupRectangles,
//      face_vision_engine.cu:1401-1539).
// Float arithmetic is written operation by operation (__fadd_rn etc.) in the
// order of the reference sources, so results equal its CPU path bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "integral.cuh"

namespace vjgb {

// Compact per-stump record: corner offsets of up to three rectangles relative
// to the window origin, the rectangle weights and the stump parameters.
struct alignas(16) DStump {
    float theta, left, right;
    int32_t nr;
    float w[3];
    int32_t pad0;
    int8_t dx[12], dy[12];  // rectangle r, corner c at [4*r + c]
    int32_t pad1[2];
};
static_assert(sizeof(DStump) == 64, "DStump is 64 bytes");

struct DStage {
    int32_t first, ntrees;
    float threshold;
    int32_t pad;
};

struct CasLevel {
    const uint32_t* sum;
    const uint64_t* sq;
    int64_t pitch;
    int workW, workH, step, scanW, scanH, tilesX;
    int64_t tileBase;
    float scale;
    int scaleIdx;
    int image;
    int pad;
};

struct ResizeJob {
    const uint8_t* src;
    int64_t srcStride;
    int srcW, srcH;
    uint8_t* dst;
    int64_t dstStride;
    int dstW, dstH;
    float sx, sy;
    int64_t itemBase;
};

struct QEntry {
    uint32_t level;
    uint32_t xy;  // (y << 16) | x, window origin in level pixels
    float inv;
    float score;
};

namespace {

constexpr int kTileW = 32, kTileH = 8;  // windows per warp tile (grid units)
constexpr int kCasWarps = 8;

// ---------------------------------------------------------------------------
// Pyramid resize, one warp per 128-pixel row chunk, 4 pixels per lane.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint8_t resize_px(const ResizeJob& J, int x, int y) {
    const float fx = __fsub_rn(__fmul_rn(__fadd_rn(static_cast<float>(x), 0.5f), J.sx), 0.5f);
    const float fy = __fsub_rn(__fmul_rn(__fadd_rn(static_cast<float>(y), 0.5f), J.sy), 0.5f);
    const int sx0 = max(0, min(static_cast<int>(floorf(fx)), J.srcW - 1));
    const int sy0 = max(0, min(static_cast<int>(floorf(fy)), J.srcH - 1));
    const int sx1 = min(sx0 + 1, J.srcW - 1);
    const int sy1 = min(sy0 + 1, J.srcH - 1);
    const float ax = __fsub_rn(fx, static_cast<float>(sx0));
    const float ay = __fsub_rn(fy, static_cast<float>(sy0));
    const uint8_t* r0 = J.src + static_cast<size_t>(sy0) * J.srcStride;
    const uint8_t* r1 = J.src + static_cast<size_t>(sy1) * J.srcStride;
    const float p00 = static_cast<float>(__ldg(r0 + sx0)), p01 = static_cast<float>(__ldg(r0 + sx1));
    const float p10 = static_cast<float>(__ldg(r1 + sx0)), p11 = static_cast<float>(__ldg(r1 + sx1));
    const float top = __fadd_rn(p00, __fmul_rn(__fsub_rn(p01, p00), ax));
    const float bot = __fadd_rn(p10, __fmul_rn(__fsub_rn(p11, p10), ax));
    const float val = __fadd_rn(top, __fmul_rn(__fsub_rn(bot, top), ay));
    const int v = __float2int_rz(__fadd_rn(val, 0.5f));
    return static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v));
}

__global__ void __launch_bounds__(256)
resize_kernel(const ResizeJob* __restrict__ jobs, int njobs, int64_t items) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t it = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; it < items; it += nw) {
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].itemBase <= it) lo = mid; else hi = mid - 1;
        }
        const ResizeJob J = jobs[lo];
        const int chunks = (J.dstW + 127) >> 7;
        const int64_t local = it - J.itemBase;
        const int y = static_cast<int>(local / chunks);
        const int x0 = static_cast<int>(local % chunks) * 128 + lane * 4;
        uint8_t* drow = J.dst + static_cast<size_t>(y) * J.dstStride;
        if (x0 + 4 <= J.dstW) {
            uchar4 v;
            v.x = resize_px(J, x0, y);
            v.y = resize_px(J, x0 + 1, y);
            v.z = resize_px(J, x0 + 2, y);
            v.w = resize_px(J, x0 + 3, y);
            *reinterpret_cast<uchar4*>(drow + x0) = v;
        } else {
            for (int i = 0; i < 4; ++i)
                if (x0 + i < J.dstW) drow[x0 + i] = resize_px(J, x0 + i, y);
        }
    }
}

// ---------------------------------------------------------------------------
// Window evaluation (face_vision_engine.cu:463-545, main.cu:755-819).
// ---------------------------------------------------------------------------

// Variance gate; returns invNorm or 0 when the window is rejected.
__device__ __forceinline__ float window_inv(const CasLevel& L, int x, int y, int winW, int winH, int normMode) {
    const int64_t P = L.pitch;
    const int nw = winW - 2, nh = winH - 2;
    const int64_t b = static_cast<int64_t>(y) * P + x;
    const int64_t o0 = b + P + 1, o1 = b + P + 1 + nw, o2 = b + (1 + nh) * P + 1, o3 = b + (1 + nh) * P + 1 + nw;
    const uint32_t s0 = __ldg(L.sum + o0), s1 = __ldg(L.sum + o1), s2 = __ldg(L.sum + o2), s3 = __ldg(L.sum + o3);
    double ns;
    if (normMode == VJ_NORM_FLOAT_CORNERS) {
        ns = static_cast<double>(
            __fadd_rn(__fsub_rn(__fsub_rn(corner_f(s0), corner_f(s1)), corner_f(s2)), corner_f(s3)));
    } else {
        ns = static_cast<double>(static_cast<int32_t>(s0 - s1 - s2 + s3));
    }
    const uint32_t q = static_cast<uint32_t>(__ldg(L.sq + o0)) - static_cast<uint32_t>(__ldg(L.sq + o1)) -
                       static_cast<uint32_t>(__ldg(L.sq + o2)) + static_cast<uint32_t>(__ldg(L.sq + o3));
    const double area = static_cast<double>(nw * nh);
    const double nf2 = __dsub_rn(__dmul_rn(area, static_cast<double>(q)), __dmul_rn(ns, ns));
    if (!(nf2 > 0.0)) return 0.0f;
    const float inv = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn(nf2)));
    if (!(__dmul_rn(area, static_cast<double>(inv)) < 1e-1)) return 0.0f;
    return inv;
}

// Value of one stump (leftVal or rightVal) for the window at level offset `b`
// (main.cu:785-797, face_vision_engine.cu:500-537).
__device__ __forceinline__ float stump_value(const DStump* __restrict__ sp, const uint32_t* __restrict__ sum, int64_t P,
                                             int64_t b, float inv) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(sp));
    const float4 wv = __ldg(reinterpret_cast<const float4*>(sp) + 1);
    const int4 d = __ldg(reinterpret_cast<const int4*>(sp) + 2);
    const int4 e = __ldg(reinterpret_cast<const int4*>(sp) + 3);
    const int nr = __float_as_int(a.w);
    const uint32_t dxw[3] = {static_cast<uint32_t>(d.x), static_cast<uint32_t>(d.y), static_cast<uint32_t>(d.z)};
    const uint32_t dyw[3] = {static_cast<uint32_t>(d.w), static_cast<uint32_t>(e.x), static_cast<uint32_t>(e.y)};
    const float wr[3] = {wv.x, wv.y, wv.z};
    float raw = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        if (r < nr) {
            float c[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int ci = 4 * r + q;
                const int dx = static_cast<int8_t>((dxw[ci >> 2] >> (8 * (ci & 3))) & 0xFFu);
                const int dy = static_cast<int8_t>((dyw[ci >> 2] >> (8 * (ci & 3))) & 0xFFu);
                c[q] = corner_f(__ldg(sum + b + dy * P + dx));
            }
            const float v = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(c[0], c[1]), c[2]), c[3]), wr[r]);
            raw = (r == 0) ? v : __fadd_rn(raw, v);
        }
    }
    return __fmul_rn(raw, inv) < a.x ? a.y : a.z;
}

// Sum of one stage's stumps, added in stump order.  Four stumps are
// evaluated before their values are added so their ~40 integral loads are in
// flight together; the additions keep the reference's order, so the sum is
// the same float.
__device__ __forceinline__ float stage_sum(const DStump* __restrict__ stumps, const DStage& st,
                                           const uint32_t* __restrict__ sum, int64_t P, int64_t b, float inv) {
    const DStump* sp = stumps + st.first;
    float acc = 0.0f;
    int k = 0;
    for (; k + 4 <= st.ntrees; k += 4) {
        const float c0 = stump_value(sp + k, sum, P, b, inv);
        const float c1 = stump_value(sp + k + 1, sum, P, b, inv);
        const float c2 = stump_value(sp + k + 2, sum, P, b, inv);
        const float c3 = stump_value(sp + k + 3, sum, P, b, inv);
        acc = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(acc, c0), c1), c2), c3);
    }
    for (; k < st.ntrees; ++k) acc = __fadd_rn(acc, stump_value(sp + k, sum, P, b, inv));
    return acc;
}

__device__ __forceinline__ void emit(const CasLevel* __restrict__ levels, const QEntry& e, int winW, int winH,
                                     vj_detection* __restrict__ out, int cap, int* __restrict__ counts, bool valid) {
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int image = valid ? __ldg(&levels[e.level].image) : -1;
    // one atomic per image present in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, image);
    int base = 0;
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) base = atomicAdd(counts + image, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!valid) return;
    const int slot = base + __popc(peers & lanemask_lt());
    if (slot < cap) {
        const float scale = __ldg(&levels[e.level].scale);
        const int x = static_cast<int>(e.xy & 0xFFFFu), y = static_cast<int>(e.xy >> 16);
        vj_detection d;
        d.x = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(x), scale), 0.5f));
        d.y = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(y), scale), 0.5f));
        d.w = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(winW), scale), 0.5f));
        d.h = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(winH), scale), 0.5f));
        d.scaleIdx = __ldg(&levels[e.level].scaleIdx);
        d.score = e.score;
        out[static_cast<size_t>(image) * cap + slot] = d;
    }
}

struct CasArgs {
    const CasLevel* levels;
    int nLevels;
    int64_t totalTiles;   // windows come from tiles of the levels when qin is null
    const QEntry* qin;    // otherwise from this queue
    const int* qinCount;
    int qinCap;
    const DStump* stumps;
    const DStage* stages;
    int s0, s1, nStages;  // this pass runs stages [s0, s1)
    int winW, winH, normMode;
    unsigned long long* workCounter;
    QEntry* qout;
    int* qoutCount;
    int qcap;
    vj_detection* dets;
    int detCap;
    int* detCounts;
};

__device__ __forceinline__ int find_level(const CasLevel* __restrict__ levels, int n, int64_t t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (levels[mid].tileBase <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Appends `valid` lanes' entries to a queue with one atomic per warp; the
// counter keeps counting past qcap so the host sees an overflow.
__device__ __forceinline__ void push_queue(QEntry* __restrict__ q, int* __restrict__ qcount, int qcap, bool valid,
                                           const QEntry& e) {
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(qcount, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (valid) {
        const int slot = base + __popc(m & lanemask_lt());
        if (slot < qcap) q[slot] = e;
    }
}

constexpr int kListCap = kTileW * kTileH;  // windows a warp holds at once

// One cascade pass.  Each warp repeatedly takes a batch of windows - a 32x8
// tile of some level (after the variance gate), or up to 256 queue entries -
// into a private list in shared memory, runs stages [s0, s1) over it 32
// windows at a time, and after every stage compacts the survivors with a
// ballot so the next stage again runs on full warps.  Survivors go to the
// next queue, or become detections after the last stage.
__global__ void __launch_bounds__(kCasWarps * 32)
cascade_kernel(CasArgs A) {
    __shared__ QEntry lst[kCasWarps][kListCap];
    const int lane = threadIdx.x & 31;
    QEntry* Lst = lst[threadIdx.x >> 5];
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(A.workCounter, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        int count = 0;
        if (A.qin == nullptr) {
            if (t >= static_cast<unsigned long long>(A.totalTiles)) break;
            const int li = find_level(A.levels, A.nLevels, static_cast<int64_t>(t));
            const CasLevel L = A.levels[li];
            const int64_t local = static_cast<int64_t>(t) - L.tileBase;
            const int tx = static_cast<int>(local % L.tilesX), ty = static_cast<int>(local / L.tilesX);
            for (int r = 0; r < kTileH; ++r) {
                const int gx = tx * kTileW + lane, gy = ty * kTileH + r;
                const int x = gx * L.step, y = gy * L.step;
                float iv = 0.0f;
                if (gx < L.scanW && gy < L.scanH) iv = window_inv(L, x, y, A.winW, A.winH, A.normMode);
                const bool ok = iv != 0.0f;
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (ok) {
                    QEntry e;
                    e.level = static_cast<uint32_t>(li);
                    e.xy = (static_cast<uint32_t>(y) << 16) | static_cast<uint32_t>(x);
                    e.inv = iv;
                    e.score = 0.0f;
                    Lst[count + __popc(m & lanemask_lt())] = e;
                }
                count += __popc(m);
            }
        } else {
            // Entries per warp: enough to keep every warp of the grid busy,
            // between 32 and the list capacity.
            const int n = min(*A.qinCount, A.qinCap);
            const int warps = gridDim.x * kCasWarps;
            const int chunk = min(kListCap, max(32, ((n + warps - 1) / warps + 31) & ~31));
            const int64_t base = static_cast<int64_t>(t) * chunk;
            if (base >= n) break;
            count = static_cast<int>(n - base < chunk ? n - base : chunk);
            for (int i = lane; i < count; i += 32) Lst[i] = A.qin[base + i];
        }
        __syncwarp();
        for (int si = A.s0; si < A.s1 && count > 0; ++si) {
            const DStage st = A.stages[si];
            int nc = 0;
            for (int g = 0; g < count; g += 32) {
                const int i = g + lane;
                const bool act = i < count;
                QEntry e{};
                float s = 0.0f;
                if (act) {
                    e = Lst[i];
                    const CasLevel* L = A.levels + e.level;
                    const int64_t P = __ldg(&L->pitch);
                    const uint32_t* sum = reinterpret_cast<const uint32_t*>(__ldg(reinterpret_cast<const unsigned long long*>(&L->sum)));
                    const int64_t b = static_cast<int64_t>(e.xy >> 16) * P + static_cast<int64_t>(e.xy & 0xFFFFu);
                    s = stage_sum(A.stumps, st, sum, P, b, e.inv);
                }
                const bool pass = act && !(s < st.threshold);
                const unsigned m = __ballot_sync(0xffffffffu, pass);
                __syncwarp();
                if (pass) {
                    e.score = s;
                    Lst[nc + __popc(m & lanemask_lt())] = e;
                }
                nc += __popc(m);
                __syncwarp();
            }
            count = nc;
        }
        for (int g = 0; g < count; g += 32) {
            const int i = g + lane;
            const bool act = i < count;
            QEntry e{};
            if (act) e = Lst[i];
            if (A.s1 >= A.nStages)
                emit(A.levels, e, A.winW, A.winH, A.dets, A.detCap, A.detCounts, act);
            else
                push_queue(A.qout, A.qoutCount, A.qcap, act, e);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap && p) return VJ_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
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
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct HBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap && p) return VJ_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        const cudaError_t e = cudaMallocHost(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return set_error(VJ_OUT_OF_MEMORY, std::string("pinned buffer: ") + cudaGetErrorString(e));
        }
        cap = want;
        return VJ_OK;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct LevelGeom {
    int scaleIdx;
    float scale;
    int w, h, step;
    int src;  // index of the level it is resized from in this image's list, -1 = original
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
            g.src = idx == 0 ? -2 : prev;  // -2: the image itself
            out.push_back(g);
            prev = static_cast<int>(out.size()) - 1;
        }
        scale *= sf;
        ++idx;
        if (idx > 100000) break;
    }
    return out;
}

int sm_count_d() {
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

}  // namespace

// Restatement of groupRectanglesCpu (face_vision_engine.cu:1401-1539):
// union-find (path compression, union by rank) over similar rectangles found
// by an x-sorted sweep, clusters with more than max(1, minNeighbors) members
// averaged with integer division, then clusters contained in a more populous
// one dropped.
std::vector<vj_detection> group_rectangles(const std::vector<vj_detection>& in, int minNeighbors, float eps) {
    const int n = static_cast<int>(in.size());
    if (n == 0) return {};
    std::vector<int> parent(n), rnk(n, 0), order(n);
    for (int i = 0; i < n; ++i) parent[i] = order[i] = i;
    auto find = [&](int x) {
        int r = x;
        while (parent[r] != r) r = parent[r];
        while (parent[x] != r) {
            const int nx = parent[x];
            parent[x] = r;
            x = nx;
        }
        return r;
    };
    auto unite = [&](int a, int b) {
        a = find(a);
        b = find(b);
        if (a == b) return;
        if (rnk[a] < rnk[b]) std::swap(a, b);
        parent[b] = a;
        if (rnk[a] == rnk[b]) ++rnk[a];
    };
    auto byX = [](const std::vector<vj_detection>& v) {
        return [&v](int a, int b) { return v[a].x != v[b].x ? v[a].x < v[b].x : a < b; };
    };
    std::sort(order.begin(), order.end(), byX(in));
    for (int oi = 0; oi < n; ++oi) {
        const vj_detection& a = in[order[oi]];
        const int reach = static_cast<int>(eps * static_cast<float>(a.w + a.h) * 0.5f);
        for (int oj = oi + 1; oj < n; ++oj) {
            const vj_detection& b = in[order[oj]];
            if (b.x - a.x > reach) break;
            const int delta = static_cast<int>(eps * static_cast<float>(std::min(a.w, b.w) + std::min(a.h, b.h)) * 0.5f);
            if (std::abs(a.x - b.x) <= delta && std::abs(a.y - b.y) <= delta &&
                std::abs(a.x + a.w - b.x - b.w) <= delta && std::abs(a.y + a.h - b.y - b.h) <= delta)
                unite(order[oi], order[oj]);
        }
    }
    struct Acc {
        int64_t x = 0, y = 0, w = 0, h = 0;
        int count = 0;
        float best = -INFINITY;
        int scaleIdx = 0;
    };
    std::vector<Acc> acc(n);
    for (int i = 0; i < n; ++i) {
        Acc& c = acc[find(i)];
        c.x += in[i].x;
        c.y += in[i].y;
        c.w += in[i].w;
        c.h += in[i].h;
        c.count += 1;
        if (in[i].score > c.best) {
            c.best = in[i].score;
            c.scaleIdx = in[i].scaleIdx;
        }
    }
    std::vector<vj_detection> cl;
    std::vector<int> cc;
    const int minN = std::max(1, minNeighbors);
    for (int i = 0; i < n; ++i) {
        if (find(i) != i || acc[i].count <= minN) continue;
        const Acc& c = acc[i];
        vj_detection d;
        d.x = static_cast<int>(c.x / c.count);
        d.y = static_cast<int>(c.y / c.count);
        d.w = static_cast<int>(c.w / c.count);
        d.h = static_cast<int>(c.h / c.count);
        d.scaleIdx = c.scaleIdx;
        d.score = c.best;
        cl.push_back(d);
        cc.push_back(c.count);
    }
    int maxW = 0;
    for (const auto& d : cl) maxW = std::max(maxW, d.w);
    std::vector<int> co(cl.size());
    for (size_t i = 0; i < cl.size(); ++i) co[i] = static_cast<int>(i);
    std::sort(co.begin(), co.end(), byX(cl));
    std::vector<vj_detection> out;
    for (size_t i = 0; i < cl.size(); ++i) {
        const vj_detection& r1 = cl[i];
        const int n1 = cc[i];
        const float lb = static_cast<float>(r1.x + r1.w) - (1.0f + eps) * static_cast<float>(maxW);
        const float rb = static_cast<float>(r1.x) + eps * static_cast<float>(maxW);
        bool drop = false;
        for (int o : co) {
            const vj_detection& r2 = cl[o];
            if (r2.x < static_cast<int>(lb)) continue;
            if (r2.x > static_cast<int>(rb)) break;
            if (static_cast<size_t>(o) == i) continue;
            const int n2 = cc[o];
            const int dx = static_cast<int>(static_cast<float>(r2.w) * eps);
            const int dy = static_cast<int>(static_cast<float>(r2.h) * eps);
            if (r1.x >= r2.x - dx && r1.y >= r2.y - dy && r1.x + r1.w <= r2.x + r2.w + dx &&
                r1.y + r1.h <= r2.y + r2.h + dy && (n2 > std::max(3, n1) || n1 < 3)) {
                drop = true;
                break;
            }
        }
        if (!drop) out.push_back(r1);
    }
    return out;
}

}  // namespace vjgb

using namespace vjgb;

struct vj_detector {
    int winW = 24, winH = 24, maxW = 0, maxH = 0, maxDet = 0;
    int normMode = VJ_NORM_FLOAT_CORNERS;
    int nStages = 0, nStumps = 0;
    std::vector<DStage> hStages;
    DBuf stumps, stages;
    // Work buffers, grown on demand.
    DBuf imgs, pix, iiSum, iiSq, totS, totQ, plan, qA, qB, dets, counts, ctrs;
    HBuf hplan, hcounts, hdets;
    // Stage schedule: the tile pass covers [0, tileStages); queue passes end
    // at passEnds.  Capacity hints carry the largest queue and per-image raw
    // detection counts seen so far, so a repeat workload needs no retry.
    int tileStages = 0;
    std::vector<int> passEnds;
    int tileStumps = 64, passStumps = 600;
    int64_t qHint = 0;
    int detHint = 0;
};

namespace {

// Stage schedule: the tile pass runs stages until it has covered tileStumps
// stumps; each queue pass then covers at least passStumps stumps (the last
// takes the rest).  At most 7 queue passes (work counters available).
void schedule_passes(vj_detector* d) {
    int acc = 0, s = 0;
    while (s < d->nStages && (acc < d->tileStumps || s == 0)) acc += d->hStages[s++].ntrees;
    d->tileStages = s;
    d->passEnds.clear();
    int remaining = 0;
    for (int k = s; k < d->nStages; ++k) remaining += d->hStages[k].ntrees;
    const int per = std::max(d->passStumps, (remaining + 6) / 7);
    while (s < d->nStages) {
        int a = 0;
        while (s < d->nStages && a < per) a += d->hStages[s++].ntrees;
        d->passEnds.push_back(s);
    }
}

struct BatchImage {
    const uint8_t* ptr;
    int w, h;
    int64_t stride;
};

int run_batch(vj_detector* D, const std::vector<BatchImage>& ims, bool onDevice, float sf, int minN, int minObj,
              int maxDet, bool group, vj_detection* out, int capPer, int* counts, cudaStream_t s) {
    const int nImg = static_cast<int>(ims.size());
    // ---- plan levels and buffers
    std::vector<std::vector<LevelGeom>> geo(nImg);
    int64_t pixBytes = 0, iiElems = 0, imgBytes = 0;
    std::vector<int64_t> imgOff(nImg, 0);
    for (int i = 0; i < nImg; ++i) {
        geo[i] = plan_levels(ims[i].w, ims[i].h, D->winW, D->winH, sf, minObj);
        if (!onDevice) {
            imgOff[i] = imgBytes;
            imgBytes += align_up(static_cast<int64_t>(ims[i].w), 16) * ims[i].h;
        }
        for (const auto& g : geo[i]) {
            if (g.src != -2) pixBytes += align_up(g.w, 16) * g.h;
            iiElems += (g.h + 1) * ii_pitch(g.w);
        }
    }
    int st;
    if (!onDevice && (st = D->imgs.ensure(imgBytes)) != VJ_OK) return st;
    if ((st = D->pix.ensure(pixBytes)) != VJ_OK) return st;
    if ((st = D->iiSum.ensure(iiElems * 4)) != VJ_OK) return st;
    if ((st = D->iiSq.ensure(iiElems * 8)) != VJ_OK) return st;

    std::vector<IIJob> iij;
    std::vector<CasLevel> lv;
    std::vector<std::vector<ResizeJob>> rj;  // by chain position
    int64_t pixOff = 0, iiOff = 0, tiles = 0, windows = 0;
    for (int i = 0; i < nImg; ++i) {
        const uint8_t* base = onDevice ? ims[i].ptr : D->imgs.as<uint8_t>() + imgOff[i];
        const int64_t baseStride = onDevice ? ims[i].stride : align_up(ims[i].w, 16);
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
                // chain position: number of resizes before this one in the image
                int pos = 0;
                for (int q = g.src; q >= 0; q = geo[i][q].src)
                    if (geo[i][q].src != -2) ++pos;
                if (static_cast<int>(rj.size()) <= pos) rj.resize(pos + 1);
                rj[pos].push_back(r);
                lp[k] = dst;
                ls[k] = dstStride;
            }
            IIJob J{};
            J.pix = lp[k];
            J.stride = ls[k];
            J.w = g.w;
            J.h = g.h;
            J.pitch = ii_pitch(g.w);
            J.sum = D->iiSum.as<uint32_t>() + iiOff;
            J.sq = D->iiSq.as<uint64_t>() + iiOff;
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
            c.tilesX = (c.scanW + kTileW - 1) / kTileW;
            c.tileBase = tiles;
            tiles += static_cast<int64_t>(c.tilesX) * ((c.scanH + kTileH - 1) / kTileH);
            windows += static_cast<int64_t>(c.scanW) * c.scanH;
            c.scale = g.scale;
            c.scaleIdx = g.scaleIdx;
            c.image = i;
            lv.push_back(c);
        }
    }
    const IIPlan ip = plan_integral_jobs(iij.data(), static_cast<int>(iij.size()));
    if ((st = D->totS.ensure(std::max<int64_t>(1, ip.totRows * ip.totPitch) * 4)) != VJ_OK) return st;
    if ((st = D->totQ.ensure(std::max<int64_t>(1, ip.totRows * ip.totPitch) * 8)) != VJ_OK) return st;
    // Queue and raw-detection capacities start from typical occupancy; the
    // counters keep counting past capacity, so an overflow is detected and the
    // call repeated with the sizes it needed.
    int qcap = static_cast<int>(
        std::min<int64_t>(std::max<int64_t>({windows / 8, int64_t(1) << 16, D->qHint}), INT32_MAX / 2));
    int detCap = std::max({64, std::min(D->maxDet, 4096), D->detHint});
    // ---- plan upload: [IIJob][CasLevel][ResizeJob...]
    std::vector<int64_t> rjOff;
    int64_t planBytes = align_up(sizeof(IIJob) * iij.size(), 64);
    const int64_t lvOff = planBytes;
    planBytes += align_up(sizeof(CasLevel) * std::max<size_t>(lv.size(), 1), 64);
    std::vector<int64_t> rjItems;
    for (auto& v : rj) {
        int64_t items = 0;
        for (auto& r : v) {
            r.itemBase = items;
            items += static_cast<int64_t>(r.dstH) * ((r.dstW + 127) / 128);
        }
        rjItems.push_back(items);
        rjOff.push_back(planBytes);
        planBytes += align_up(sizeof(ResizeJob) * v.size(), 64);
    }
    if ((st = D->plan.ensure(planBytes)) != VJ_OK) return st;
    if ((st = D->hplan.ensure(planBytes)) != VJ_OK) return st;
    char* hp = D->hplan.as<char>();
    std::memcpy(hp, iij.data(), sizeof(IIJob) * iij.size());
    std::memcpy(hp + lvOff, lv.data(), sizeof(CasLevel) * lv.size());
    for (size_t k = 0; k < rj.size(); ++k) std::memcpy(hp + rjOff[k], rj[k].data(), sizeof(ResizeJob) * rj[k].size());
    if ((st = D->counts.ensure(sizeof(int) * (nImg + 4))) != VJ_OK) return st;
    if ((st = D->ctrs.ensure(64)) != VJ_OK) return st;
    if ((st = D->hcounts.ensure(sizeof(int) * (nImg + 4))) != VJ_OK) return st;

    for (int attempt = 0; attempt < 3; ++attempt) {
        if ((st = D->dets.ensure(sizeof(vj_detection) * static_cast<size_t>(detCap) * nImg)) != VJ_OK) return st;
        if ((st = D->qA.ensure(sizeof(QEntry) * static_cast<size_t>(qcap))) != VJ_OK) return st;
        if ((st = D->qB.ensure(sizeof(QEntry) * static_cast<size_t>(qcap))) != VJ_OK) return st;
        char* dp = D->plan.as<char>();
        VJ_CUDA_TRY(cudaMemcpyAsync(dp, hp, planBytes, cudaMemcpyHostToDevice, s));
        if (!onDevice)
            for (int i = 0; i < nImg; ++i)
                VJ_CUDA_TRY(cudaMemcpy2DAsync(D->imgs.as<uint8_t>() + imgOff[i], align_up(ims[i].w, 16), ims[i].ptr,
                                              ims[i].stride, ims[i].w, ims[i].h, cudaMemcpyHostToDevice, s));
        for (size_t k = 0; k < rj.size(); ++k) {
            const int64_t items = rjItems[k];
            const int grid = static_cast<int>(std::min<int64_t>((items + 7) / 8, 16LL * sm_count_d()));
            VJ_TIMED_LAUNCH("resize_kernel", s,
                            resize_kernel<<<std::max(grid, 1), 256, 0, s>>>(
                                reinterpret_cast<const ResizeJob*>(dp + rjOff[k]), static_cast<int>(rj[k].size()),
                                items));
            VJ_LAUNCH_CHECK("resize_kernel");
        }
        st = launch_integral_jobs(reinterpret_cast<const IIJob*>(dp), static_cast<int>(iij.size()), ip,
                                  D->totS.as<uint32_t>(), D->totQ.as<uint64_t>(), s);
        if (st != VJ_OK) return st;
        VJ_CUDA_TRY(cudaMemsetAsync(D->counts.p, 0, sizeof(int) * (nImg + 4), s));
        VJ_CUDA_TRY(cudaMemsetAsync(D->ctrs.p, 0, 64, s));
        int* qCount = D->counts.as<int>() + nImg;  // two queue counters after the image counts
        const CasLevel* dLv = reinterpret_cast<const CasLevel*>(dp + lvOff);
        unsigned long long* ctr = D->ctrs.as<unsigned long long>();  // one work counter per pass
        CasArgs ca{};
        ca.levels = dLv;
        ca.nLevels = static_cast<int>(lv.size());
        ca.totalTiles = tiles;
        ca.qin = nullptr;
        ca.stumps = D->stumps.as<DStump>();
        ca.stages = D->stages.as<DStage>();
        ca.s0 = 0;
        ca.s1 = D->tileStages;
        ca.nStages = D->nStages;
        ca.winW = D->winW;
        ca.winH = D->winH;
        ca.normMode = D->normMode;
        ca.workCounter = ctr;
        ca.qout = D->qA.as<QEntry>();
        ca.qoutCount = qCount;
        ca.qcap = qcap;
        ca.dets = D->dets.as<vj_detection>();
        ca.detCap = detCap;
        ca.detCounts = D->counts.as<int>();
        const int casGrid = sm_count_d() * 8;
        static const char* const kPassName[8] = {"cascade_kernel(tiles)", "cascade_kernel(pass1)",
                                                 "cascade_kernel(pass2)", "cascade_kernel(pass3)",
                                                 "cascade_kernel(pass4)", "cascade_kernel(pass5)",
                                                 "cascade_kernel(pass6)", "cascade_kernel(pass7)"};
        if (tiles > 0) {
            VJ_TIMED_LAUNCH(kPassName[0], s, cascade_kernel<<<casGrid, kCasWarps * 32, 0, s>>>(ca));
            VJ_LAUNCH_CHECK("cascade_kernel");
        }
        QEntry* qin = D->qA.as<QEntry>();
        QEntry* qout = D->qB.as<QEntry>();
        int* cin = qCount;
        int* cout = qCount + 1;
        for (size_t p = 0; p < D->passEnds.size(); ++p) {
            VJ_CUDA_TRY(cudaMemsetAsync(cout, 0, sizeof(int), s));
            CasArgs qa = ca;
            qa.qin = qin;
            qa.qinCount = cin;
            qa.qinCap = qcap;
            qa.s0 = p == 0 ? D->tileStages : D->passEnds[p - 1];
            qa.s1 = D->passEnds[p];
            qa.workCounter = ctr + 1 + p;
            qa.qout = qout;
            qa.qoutCount = cout;
            VJ_TIMED_LAUNCH(kPassName[std::min<size_t>(p + 1, 7)], s,
                            cascade_kernel<<<casGrid, kCasWarps * 32, 0, s>>>(qa));
            VJ_LAUNCH_CHECK("cascade_kernel");
            std::swap(qin, qout);
            std::swap(cin, cout);
        }
        VJ_CUDA_TRY(cudaMemcpyAsync(D->hcounts.p, D->counts.p, sizeof(int) * (nImg + 2), cudaMemcpyDeviceToHost, s));
        VJ_CUDA_TRY(cudaStreamSynchronize(s));
        const int* hc = D->hcounts.as<int>();
        int need = 0, qneed = 0;
        for (int i = 0; i < nImg; ++i) need = std::max(need, hc[i]);
        qneed = std::max(hc[nImg], hc[nImg + 1]);
        D->qHint = std::max<int64_t>(D->qHint, qneed + qneed / 4);
        D->detHint = std::max(D->detHint, need + need / 4);
        if (qneed > qcap || need > detCap) {
            qcap = std::max(qcap, qneed);
            detCap = std::max(detCap, need);
            continue;
        }
        // ---- results
        if ((st = D->hdets.ensure(sizeof(vj_detection) * static_cast<size_t>(detCap) * nImg)) != VJ_OK) return st;
        for (int i = 0; i < nImg; ++i)
            if (hc[i] > 0)
                VJ_CUDA_TRY(cudaMemcpyAsync(D->hdets.as<vj_detection>() + static_cast<size_t>(i) * detCap,
                                            D->dets.as<vj_detection>() + static_cast<size_t>(i) * detCap,
                                            sizeof(vj_detection) * std::min(hc[i], detCap), cudaMemcpyDeviceToHost, s));
        VJ_CUDA_TRY(cudaStreamSynchronize(s));
        const int limit = std::max(1, maxDet);
        auto post = [&](int i) {
            const vj_detection* src = D->hdets.as<vj_detection>() + static_cast<size_t>(i) * detCap;
            std::vector<vj_detection> raw(src, src + std::min(hc[i], detCap));
            std::sort(raw.begin(), raw.end(), [](const vj_detection& a, const vj_detection& b) {
                if (a.scaleIdx != b.scaleIdx) return a.scaleIdx < b.scaleIdx;
                if (a.y != b.y) return a.y < b.y;
                return a.x < b.x;
            });
            if (static_cast<int>(raw.size()) > limit) raw.resize(limit);
            std::vector<vj_detection> res = group ? group_rectangles(raw, minN, 0.2f) : std::move(raw);
            const int k = std::min(static_cast<int>(res.size()), capPer);
            if (k > 0) std::memcpy(out + static_cast<size_t>(i) * capPer, res.data(), sizeof(vj_detection) * k);
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
        return VJ_OK;
    }
    return set_error(VJ_RUNTIME_ERROR, "detection buffer overflow");
}

}  // namespace

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
    for (DBuf* b : {&d->stumps, &d->stages, &d->imgs, &d->pix, &d->iiSum, &d->iiSq, &d->totS, &d->totQ, &d->plan,
                    &d->qA, &d->qB, &d->dets, &d->counts, &d->ctrs})
        b->release();
    d->hplan.release();
    d->hcounts.release();
    d->hdets.release();
    delete d;
    return ok();
}

int vj_detector_clear_model(vj_detector* d) {
    if (!d) return set_error(VJ_INVALID_ARG, "vj_detector_clear_model: null detector");
    d->stumps.release();
    d->stages.release();
    d->nStages = d->nStumps = 0;
    d->hStages.clear();
    return ok();
}

int vj_detector_set_model(vj_detector* d, const vj_haar_feature* features, int64_t featureCount,
                          const vj_stump4* stumps, int64_t stumpCount, const vj_cascade_stage* stages,
                          int64_t stageCount) {
    if (!d || !features || !stumps || !stages || featureCount <= 0 || stumpCount <= 0 || stageCount <= 0 ||
        stumpCount > INT32_MAX || stageCount > INT32_MAX)
        return set_error(VJ_INVALID_ARG, "vj_detector_set_model: bad arguments");
    const int mW = d->winW + 1;
    std::vector<DStump> ds(static_cast<size_t>(stumpCount));
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
        for (int r = 0; r < 3; ++r) {
            o.w[r] = rr[r]->w;
            const int32_t p[4] = {rr[r]->p0, rr[r]->p1, rr[r]->p2, rr[r]->p3};
            for (int c = 0; c < 4; ++c) {
                // BuildFeatureLUTKernel's decode (face_vision_engine.cu:360-365).
                const int dy = p[c] / mW, dx = p[c] - dy * mW;
                if (r < o.nr && (dx < 0 || dx > d->winW || dy < 0 || dy > d->winH))
                    return set_error(VJ_INVALID_ARG, "vj_detector_set_model: feature corner outside the window");
                o.dx[4 * r + c] = static_cast<int8_t>(r < o.nr ? dx : 0);
                o.dy[4 * r + c] = static_cast<int8_t>(r < o.nr ? dy : 0);
            }
        }
    }
    std::vector<DStage> dst(static_cast<size_t>(stageCount));
    for (int64_t i = 0; i < stageCount; ++i) {
        if (stages[i].ntrees < 0 || stages[i].first < 0 ||
            static_cast<int64_t>(stages[i].first) + stages[i].ntrees > stumpCount)
            return set_error(VJ_INVALID_ARG, "vj_detector_set_model: stage outside the stump array");
        dst[static_cast<size_t>(i)] = DStage{stages[i].first, stages[i].ntrees, stages[i].threshold, 0};
    }
    int st;
    if ((st = d->stumps.ensure(sizeof(DStump) * ds.size())) != VJ_OK) return st;
    if ((st = d->stages.ensure(sizeof(DStage) * dst.size())) != VJ_OK) return st;
    VJ_CUDA_TRY(cudaMemcpy(d->stumps.p, ds.data(), sizeof(DStump) * ds.size(), cudaMemcpyHostToDevice));
    VJ_CUDA_TRY(cudaMemcpy(d->stages.p, dst.data(), sizeof(DStage) * dst.size(), cudaMemcpyHostToDevice));
    d->nStages = static_cast<int>(stageCount);
    d->nStumps = static_cast<int>(stumpCount);
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
    std::vector<BatchImage> ims(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        if (!images[i] || w[i] <= 0 || h[i] <= 0 || stride[i] < w[i] || w[i] > d->maxW || h[i] > d->maxH)
            return set_error(VJ_INVALID_ARG, "vj_detect_batch: bad image " + std::to_string(i));
        ims[static_cast<size_t>(i)] = BatchImage{images[i], w[i], h[i], stride[i]};
        counts[i] = 0;
    }
    const int maxDet = std::max(1, std::min(maxDetectionsPerImage, d->maxDet));
    const int st = run_batch(d, ims, images_on_device != 0, scaleFactor, minNeighbors, minObjectSize, maxDet,
                             applyGrouping != 0, out, capPerImage, counts, static_cast<cudaStream_t>(stream));
    return st == VJ_OK ? ok() : st;
}

}  // extern "C"
