// Device side of multiscale cascade detection: the records the detection
// kernel reads, the window arithmetic, and the phases of the persistent
// detection kernel.
//
// Window arithmetic follows the reference operation by operation
// (src/face_vision_engine.cu:463-545 and its CPU twin src/main.cu:755-819):
// float corners, (p0 - p1 - p2 + p3) * w per rectangle added in rectangle
// order, raw * invNorm compared with theta, leaf values added in stump order
// starting from 0.0f.  With --fmad=false and explicit __fadd_rn etc. the
// results equal the reference CPU path bit for bit.
#pragma once

#include <climits>
#include <type_traits>

#include "group_dev.cuh"
#include "integral_dev.cuh"

namespace vjgb {

// Stump record for per-lane global gathers (lane-per-window passes): corner
// offsets of up to three rectangles relative to the window origin.
struct alignas(16) DStump {
    float theta, left, right;
    int32_t nr;
    float w[3];
    int32_t pad0;
    int8_t dx[12], dy[12];  // rectangle r, corner c at [4*r + c]
    int32_t pad1[2];
};
static_assert(sizeof(DStump) == 64, "DStump is 64 bytes");

// Stump record for the warp-per-window deep pass, stored as three 16-byte
// planes (structure of arrays) so that lanes reading consecutive stumps read
// consecutive 16-byte words:
//   A = {theta, left, right, w0}, B = {w1, w2, o01, o23}, C = {o45, o67, o89, o1011}
// where oXY packs the offsets of corners X (low half) and Y (high half) into
// the window's (winW+1) x (winH+1) integral patch - the feature's own p0..p3
// indices (FastRect, common_types.cuh:26-35).  A 2-rectangle feature has
// w2 == 0 and its third rectangle is not evaluated; for a 3-rectangle feature
// with w2 == 0 skipping it is also exact, because adding the signed zero v2
// can only flip the sign of a zero raw, which compares equal.
struct PStumpPlanes {
    const uint4* a;
    const uint4* b;
    const uint4* c;
};

struct DStage {
    int32_t first, ntrees;
    float threshold;
    // Bound on |any summation of the stage's leaf values - their exact sum|
    // plus the same for the sequential FP32 sum (see deep_pass).
    float tol;
};

// One pyramid level of one image, as scanned.
struct CasLevel {
    const uint32_t* sum;
    const uint32_t* sq;  // squared sums modulo 2^32 (integral.cuh IIJobT)
    int64_t pitch;
    int workW, workH, step, scanW, scanH, tilesX;
    int64_t tileBase;
    float scale;
    int scaleIdx;
    int image;
    int pad;
};

// Level k of an image is resized from level k-1 (or the image).
struct ResizeJob {
    const uint8_t* src;
    int64_t srcStride;
    int srcW, srcH;
    uint8_t* dst;
    int64_t dstStride;
    int dstW, dstH;
    float sx, sy;
    int64_t itemBase;  // first work item (one warp per 128-pixel row chunk)
};

struct QEntry {
    uint32_t level;
    uint32_t xy;  // (y << 16) | x, window origin in level pixels
    float inv;
    float score;
};

constexpr int kCasThreads = 256;
constexpr int kCasWarps = kCasThreads / 32;
constexpr int kMaxQueuePasses = 6;
constexpr int kQueues = kMaxQueuePasses + 2;
constexpr int kPhaseStamps = 8;

// Control block, zeroed before every launch and copied to the host after it.
struct GridSync {
    unsigned int arrive;
    unsigned int error;  // set when a barrier wait ran out of time
    unsigned int pad[2];
    unsigned long long stamp[kPhaseStamps];  // %globaltimer at phase ends (block 0)
};
struct CtrlHead {
    GridSync sync;
    unsigned long long work[kQueues + 2];  // dynamic work counters of the passes
    unsigned long long stats[4];           // [0] gated windows, [1] stump evaluations
    int qcount[kQueues];                   // entries pushed to queue k (keeps counting past qcap)
    int compactTotal;                      // raw detections kept (copied to the host buffer, or grouped)
    int compactOverflow;
    int rawTotal;                          // raw detections held on the device
    int grpOverflow;                       // the grouping arrays have fewer slots than compactTotal
    int grpError;                          // a union-find retry bound ran out
    int clTotal;                           // clusters listed by the grouping (all images)
    // followed by int counts[imageCap] (raw detections per image, counting
    // past detCap), int offsets[imageCap] (start of image i's kept raw
    // detections, in the host buffer and in the grouping slots), int
    // rawOff[imageCap] (start of image i's raw detections in flat order), int
    // ccount[imageCap] (clusters of image i), int gcount[imageCap] (grouped
    // detections of image i) and uint64 selKey[imageCap] (largest canonical key
    // kept of image i)
};

// Everything the persistent kernel reads: written by the host into pinned
// memory and copied to the device by the first node of the launch graph.
struct DevPlan {
    int nImg, nLevels, nResize, nQueuePasses;
    int winW, winH, normMode, nStages;
    int tileStages, deepFrom, qcap, detCap;
    int queueEnd[kMaxQueuePasses];  // stage range of queue pass m: [m ? queueEnd[m-1] : tileStages, queueEnd[m])
    int hostCap;
    int spreadStumps;  // 1: deep-pass records reordered within blocks (detect.cu spread_banks)
    int colWalk;       // integral column pass: 1 one walk per column chunk, 0 segment totals + scan
    // Wait tests: when >= 0, this block leaves before the first grid barrier,
    // so the others' wait runs out after barrierTimeoutNs.
    int holdBlock;
    unsigned long long barrierTimeoutNs;  // 0 = kBarrierTimeoutNs
    int64_t totalTiles;
    IIPlan ip;
    const int* rjFirst;         // nResize + 1: resize jobs of chain position p
    const int64_t* rjItems;     // nResize: work items of chain position p
    const ResizeJob* rjobs;
    const IIJob32* iijobs;      // one per level
    const CasLevel* levels;
    uint32_t* totS;             // segment totals of the column passes (colWalk 0)
    uint32_t* totQ;
    const DStump* stumps;
    PStumpPlanes pstumps;
    const DStage* stages;
    QEntry* q[2];
    vj_detection* dets;         // nImg * detCap, image i at dets + i * detCap
    CtrlHead* ctrl;
    int* counts;                // in the control block
    int* offsets;               // in the control block
    int* rawOff;                // in the control block
    int* ccount;                // in the control block
    int* gcount;                // in the control block
    unsigned long long* selKey; // in the control block
    vj_detection* hostDets;     // host-mapped, hostCap entries
    GroupPlan grp;
};

// ---------------------------------------------------------------------------
// Small device helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

constexpr unsigned long long kBarrierTimeoutNs = 60ull * 1000 * 1000 * 1000;  // 60 s
constexpr unsigned kBarrierMaxSpins = 1u << 30;

// Grid-wide barrier of the cooperative launch.  Every block arrives once per
// barrier on a monotonic counter; the wait is bounded by time and by spin
// count, after which the error flag is set.  Returns false (in every thread of
// the block) once any block has set the error flag, so all blocks leave the
// kernel instead of waiting again.
__device__ __forceinline__ bool grid_barrier(GridSync* g, unsigned& epoch, unsigned long long timeoutNs) {
    __shared__ int okShared;
    __syncthreads();
    ++epoch;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&g->arrive, 1u);
        const unsigned target = epoch * gridDim.x;
        const unsigned long long t0 = global_ns();
        bool ok = true;
        // one load per spin; the error flag and the time limit are checked
        // every 32 spins
        for (unsigned it = 0;; ++it) {
            if (ld_acquire_u32(&g->arrive) >= target) break;
            if ((it & 31u) == 31u) {
                if (ld_acquire_u32(&g->error) != 0u) {
                    ok = false;
                    break;
                }
                if (global_ns() - t0 > timeoutNs || it > kBarrierMaxSpins) {
                    atomicExch(&g->error, 1u);
                    ok = false;
                    break;
                }
            }
            __nanosleep(32);
        }
        if (ok && ld_acquire_u32(&g->error) != 0u) ok = false;
        __threadfence();
        okShared = ok ? 1 : 0;
    }
    __syncthreads();
    __threadfence();
    return okShared != 0;
}

// ---------------------------------------------------------------------------
// Pyramid resize (face_vision_engine.cu:270-308, main.cu:545-585): pixel-centre
// bilinear with the reference's rounding, one warp per 128-pixel row chunk.
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
    const float p00 = static_cast<float>(r0[sx0]), p01 = static_cast<float>(r0[sx1]);
    const float p10 = static_cast<float>(r1[sx0]), p11 = static_cast<float>(r1[sx1]);
    const float top = __fadd_rn(p00, __fmul_rn(__fsub_rn(p01, p00), ax));
    const float bot = __fadd_rn(p10, __fmul_rn(__fsub_rn(p11, p10), ax));
    const float val = __fadd_rn(top, __fmul_rn(__fsub_rn(bot, top), ay));
    const int v = __float2int_rz(__fadd_rn(val, 0.5f));
    return static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v));
}

__device__ __forceinline__ void resize_item(const ResizeJob* __restrict__ jobs, int njobs, int64_t it, int lane) {
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

// ---------------------------------------------------------------------------
// Window evaluation.
// ---------------------------------------------------------------------------

// float(1 / sqrt(x)) with the reference's rounding - the double square root,
// then the double reciprocal, then the float conversion - for integer x in
// [1, 2^42).  One Newton step in double from the float reciprocal square root
// gives y within 2^-42 (relative) of 1/sqrt(x): rsqrtf is within 2 ulp
// (2^-22) and float(x) within 2^-24, so the step's error is about
// 1.5 * (2^-21.8)^2 plus a few double roundings.  The reference's double value
// is within 2^-52 of 1/sqrt(x), so the two are less than 2^11 units of y's
// last place apart, and both round to the same float unless a float rounding
// boundary lies between them: the 29 bits below float precision of y are
// then within 2^11 of the halfway pattern 2^28.  Whenever they are within
// 2^16 of it (about one value in 4000) the double square root and reciprocal
// are used instead.
__device__ __forceinline__ float inv_sqrt_as_reference(double x) {
    const double y = static_cast<double>(rsqrtf(__double2float_rn(x)));
    const double y1 = __dmul_rn(y, __dsub_rn(1.5, __dmul_rn(__dmul_rn(0.5, x), __dmul_rn(y, y))));
    const int low = static_cast<int>(static_cast<unsigned long long>(__double_as_longlong(y1)) & 0x1FFFFFFFull);
    if (abs(low - 0x10000000) > 0x10000) return __double2float_rn(y1);
    return __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn(x)));
}

// Variance gate (face_vision_engine.cu:463-492); returns invNorm, or 0 when
// the window is rejected.
__device__ __forceinline__ float window_inv(const CasLevel& L, int x, int y, int winW, int winH, int normMode) {
    const int64_t P = L.pitch;
    const int nw = winW - 2, nh = winH - 2;
    const int64_t b = static_cast<int64_t>(y) * P + x;
    const int64_t o0 = b + P + 1, o1 = b + P + 1 + nw, o2 = b + (1 + nh) * P + 1, o3 = b + (1 + nh) * P + 1 + nw;
    const uint32_t s0 = L.sum[o0], s1 = L.sum[o1], s2 = L.sum[o2], s3 = L.sum[o3];
    double ns;
    if (normMode == VJ_NORM_FLOAT_CORNERS) {
        ns = static_cast<double>(
            __fadd_rn(__fsub_rn(__fsub_rn(corner_f(s0), corner_f(s1)), corner_f(s2)), corner_f(s3)));
    } else {
        ns = static_cast<double>(static_cast<int32_t>(s0 - s1 - s2 + s3));
    }
    const uint32_t q = L.sq[o0] - L.sq[o1] - L.sq[o2] + L.sq[o3];
    const double area = static_cast<double>(nw * nh);
    const double nf2 = __dsub_rn(__dmul_rn(area, static_cast<double>(q)), __dmul_rn(ns, ns));
    if (!(nf2 > 0.0)) return 0.0f;
    const float inv = inv_sqrt_as_reference(nf2);  // nf2: an integer in [1, 2^42)
    if (!(__dmul_rn(area, static_cast<double>(inv)) < 1e-1)) return 0.0f;
    return inv;
}

// Leaf value of one stump for the window at level offset `b`, corners
// gathered from the level's integral image (main.cu:785-797).
__device__ __forceinline__ float stump_value(const DStump* __restrict__ sp, const uint32_t* sum, int64_t P, int64_t b,
                                             float inv) {
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
                c[q] = corner_f(sum[b + dy * P + dx]);
            }
            const float v = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(c[0], c[1]), c[2]), c[3]), wr[r]);
            raw = (r == 0) ? v : __fadd_rn(raw, v);
        }
    }
    return __fmul_rn(raw, inv) < a.x ? a.y : a.z;
}

// Sum of one stage's stumps for one window, added in stump order.  Four
// stumps are evaluated before their values are added so their integral loads
// are in flight together; the additions keep the reference's order.
__device__ __forceinline__ float stage_sum(const DStump* __restrict__ stumps, const DStage& st, const uint32_t* sum,
                                           int64_t P, int64_t b, float inv) {
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

// A stump decoded for one level: corner offsets dy * pitch + dx relative to
// the window origin, weights, rectangle count, threshold and leaf values.
struct LevelStump {
    int off[12];
    float w[3];
    int nr;
    float theta, left, right;
};

__device__ __forceinline__ void decode_stump(const DStump* __restrict__ sp, int pitch, LevelStump& d) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(sp));
    const float4 wv = __ldg(reinterpret_cast<const float4*>(sp) + 1);
    const int4 dd = __ldg(reinterpret_cast<const int4*>(sp) + 2);
    const int4 ee = __ldg(reinterpret_cast<const int4*>(sp) + 3);
    d.theta = a.x;
    d.left = a.y;
    d.right = a.z;
    d.nr = __float_as_int(a.w);
    d.w[0] = wv.x;
    d.w[1] = wv.y;
    d.w[2] = wv.z;
    const uint32_t dxw[3] = {static_cast<uint32_t>(dd.x), static_cast<uint32_t>(dd.y), static_cast<uint32_t>(dd.z)};
    const uint32_t dyw[3] = {static_cast<uint32_t>(dd.w), static_cast<uint32_t>(ee.x), static_cast<uint32_t>(ee.y)};
#pragma unroll
    for (int ci = 0; ci < 12; ++ci) {
        const int dx = static_cast<int8_t>((dxw[ci >> 2] >> (8 * (ci & 3))) & 0xFFu);
        const int dy = static_cast<int8_t>((dyw[ci >> 2] >> (8 * (ci & 3))) & 0xFFu);
        d.off[ci] = dy * pitch + dx;
    }
}

// Leaf value of a decoded stump for the window at integral offset b; the same
// operations in the same order as stump_value.
__device__ __forceinline__ float decoded_value(const LevelStump& d, const uint32_t* sum, int b, float inv) {
    float raw = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        if (r < d.nr) {
            const float c0 = corner_f(sum[b + d.off[4 * r]]), c1 = corner_f(sum[b + d.off[4 * r + 1]]);
            const float c2 = corner_f(sum[b + d.off[4 * r + 2]]), c3 = corner_f(sum[b + d.off[4 * r + 3]]);
            const float v = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(c0, c1), c2), c3), d.w[r]);
            raw = (r == 0) ? v : __fadd_rn(raw, v);
        }
    }
    return __fmul_rn(raw, inv) < d.theta ? d.left : d.right;
}

// Corners that a decoded stump's rectangles share (equal offsets), the
// shapes of corner_sharing: 1 (2 rects, r1.p1 = r0.p1, r1.p3 = r0.p3),
// 2 (2 rects, r1.p2 = r0.p2, r1.p3 = r0.p3), 3 (3 rects, r1.p0 = r0.p0,
// r2.p0 = r1.p3, r2.p3 = r0.p3), 0 otherwise.
__device__ __forceinline__ int decoded_sharing(const LevelStump& d) {
    if (d.nr == 2) {
        if (d.off[5] == d.off[1] && d.off[7] == d.off[3]) return 1;
        if (d.off[6] == d.off[2] && d.off[7] == d.off[3]) return 2;
    } else if (d.nr == 3) {
        if (d.off[4] == d.off[0] && d.off[8] == d.off[7] && d.off[11] == d.off[3]) return 3;
    }
    return 0;
}

// decoded_value for a stump of decoded_sharing shape S: each shared corner
// gathered once, the same operations in the same order.
template <int S>
__device__ __forceinline__ float decoded_value_shared(const LevelStump& d, const uint32_t* sum, int b, float inv) {
    if (S == 0) return decoded_value(d, sum, b, inv);
    auto ld = [&](int q) { return corner_f(sum[b + d.off[q]]); };
    auto rect = [](float c0, float c1, float c2, float c3, float w) {
        return __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(c0, c1), c2), c3), w);
    };
    const float a0 = ld(0), a1 = ld(1), a2 = ld(2), a3 = ld(3);
    float raw;
    if (S == 1) {
        const float b0 = ld(4), b2 = ld(6);
        raw = __fadd_rn(rect(a0, a1, a2, a3, d.w[0]), rect(b0, a1, b2, a3, d.w[1]));
    } else if (S == 2) {
        const float b0 = ld(4), b1 = ld(5);
        raw = __fadd_rn(rect(a0, a1, a2, a3, d.w[0]), rect(b0, b1, a2, a3, d.w[1]));
    } else {
        const float b1 = ld(5), b2 = ld(6), b3 = ld(7), e1 = ld(9), e2 = ld(10);
        raw = __fadd_rn(rect(a0, a1, a2, a3, d.w[0]), rect(a0, b1, b2, b3, d.w[1]));
        raw = __fadd_rn(raw, rect(b3, e1, e2, a3, d.w[2]));
    }
    return __fmul_rn(raw, inv) < d.theta ? d.left : d.right;
}

// Leaf value of stump k from the window's integral patch in shared memory
// (corners already converted to float; element o at patch[PS * o]).  m0
// masks the first offset: 0x3FF when the record's bits 10-15 of that half
// hold its position in the stage's block before reordering (detect.cu
// spread_banks), else 0xFFFF.
template <int PS>
__device__ __forceinline__ float patch_stump_value(const PStumpPlanes& ps, int k, const float* patch, float inv,
                                                   uint32_t m0) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(ps.a + k));
    const uint4 b = __ldg(ps.b + k);
    const uint4 c = __ldg(ps.c + k);
    const float w1 = __uint_as_float(b.x), w2 = __uint_as_float(b.y);
    // A corner at the same offset as an earlier one (the shapes of
    // corner_sharing: r1.p0 = r0.p0, r1.p1 = r0.p1, r1.p2 = r0.p2,
    // r1.p3 = r0.p3, r2.p0 = r1.p3, r2.p3 = r0.p3) takes that corner's value
    // instead of a second shared-memory read; the values are the same.
    const uint32_t o0 = b.z & m0, o1 = b.z >> 16, o2 = b.w & 0xFFFFu, o3 = b.w >> 16;
    const uint32_t o4 = c.x & 0xFFFFu, o5 = c.x >> 16, o6 = c.y & 0xFFFFu, o7 = c.y >> 16;
    auto at = [&](uint32_t o) { return patch[PS * o]; };
    const float p0 = at(o0), p1 = at(o1), p2 = at(o2), p3 = at(o3);
    float p4, p5, p6, p7;
    if (o4 == o0) p4 = p0; else p4 = at(o4);
    if (o5 == o1) p5 = p1; else p5 = at(o5);
    if (o6 == o2) p6 = p2; else p6 = at(o6);
    if (o7 == o3) p7 = p3; else p7 = at(o7);
    const float v0 = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(p0, p1), p2), p3), a.w);
    const float v1 = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(p4, p5), p6), p7), w1);
    float raw = __fadd_rn(v0, v1);
    if (w2 != 0.0f) {
        const uint32_t o8 = c.z & 0xFFFFu, o9 = c.z >> 16, o10 = c.w & 0xFFFFu, o11 = c.w >> 16;
        float p8, p11;
        if (o8 == o7) p8 = p7; else p8 = at(o8);
        if (o11 == o3) p11 = p3; else p11 = at(o11);
        const float v2 = __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(p8, at(o9)), at(o10)), p11), w2);
        raw = __fadd_rn(raw, v2);
    }
    return __fmul_rn(raw, inv) < a.x ? a.y : a.z;
}

// Output record of a window (face_vision_engine.cu:559-567): level
// coordinates scaled by the level's scale and rounded as the reference does.
__device__ __forceinline__ vj_detection make_detection(const CasLevel& L, const QEntry& e, int winW, int winH,
                                                       float score) {
    const int x = static_cast<int>(e.xy & 0xFFFFu), y = static_cast<int>(e.xy >> 16);
    vj_detection d;
    d.x = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(x), L.scale), 0.5f));
    d.y = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(y), L.scale), 0.5f));
    d.w = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(winW), L.scale), 0.5f));
    d.h = __float2int_rz(__fadd_rn(__fmul_rn(static_cast<float>(winH), L.scale), 0.5f));
    d.scaleIdx = L.scaleIdx;
    d.score = score;
    return d;
}

// Warp-wide emission of the valid lanes' windows: one atomic per image
// present in the warp; the per-image counters keep counting past detCap so
// the host sees an overflow.
__device__ __forceinline__ void emit_warp(const DevPlan& P, const QEntry& e, bool valid) {
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int image = valid ? P.levels[e.level].image : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, image);
    int base = 0;
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) base = atomicAdd(P.counts + image, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!valid) return;
    const int slot = base + __popc(peers & lanemask_lt());
    if (slot < P.detCap)
        P.dets[static_cast<size_t>(image) * P.detCap + slot] = make_detection(P.levels[e.level], e, P.winW, P.winH, e.score);
}

// Appends the valid lanes' entries to a queue with one atomic per warp.
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

__device__ __forceinline__ int find_level(const CasLevel* __restrict__ levels, int n, int64_t t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (levels[mid].tileBase <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Lane-per-window pass.  Each warp repeatedly takes a batch of windows - a
// 32 x TH tile of window positions of some level (after the variance gate) in
// the tile pass, or a chunk of queue entries in a queue pass - into a private
// list in shared memory, runs stages [s0, s1) over it 32 windows at a time,
// and after every stage compacts the survivors with a ballot, so the next
// stage again runs on full warps.  Survivors go to the next queue, or become
// detections when s1 is the last stage.  A tile's windows share their level,
// so its list holds 8-byte entries (position; the reciprocal norm, or the
// score after the last stage) and 32 * TH of them fit the 16 * TH queue
// entries of a queue pass: the lists never take more shared memory than the
// deep pass, whatever TH.
// ---------------------------------------------------------------------------
template <int TH>
__device__ __forceinline__ void lane_pass(const DevPlan& P, QEntry* lst, const QEntry* qin, int qinCount, int s0,
                                          int s1, unsigned long long* workCounter, QEntry* qout, int* qoutCount,
                                          unsigned long long& gated, unsigned long long& evals) {
    constexpr int kCapQ = 16 * TH;  // queue entries a list holds
    uint2* tl = reinterpret_cast<uint2*>(lst);  // tile entries: (y << 16 | x, inv or score bits)
    const int lane = threadIdx.x & 31;
    const bool last = s1 >= P.nStages;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(workCounter, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        int count = 0;
        int tileLevel = -1;  // the level of every window in the list (tile pass)
        if (qin == nullptr) {
            if (t >= static_cast<unsigned long long>(P.totalTiles)) break;
            const int li = find_level(P.levels, P.nLevels, static_cast<int64_t>(t));
            tileLevel = li;
            const CasLevel L = P.levels[li];
            const int64_t local = static_cast<int64_t>(t) - L.tileBase;
            const int tx = static_cast<int>(local % L.tilesX), ty = static_cast<int>(local / L.tilesX);
            for (int r = 0; r < TH; ++r) {
                const int gx = tx * 32 + lane, gy = ty * TH + r;
                const int x = gx * L.step, y = gy * L.step;
                float iv = 0.0f;
                if (gx < L.scanW && gy < L.scanH) iv = window_inv(L, x, y, P.winW, P.winH, P.normMode);
                const bool ok = iv != 0.0f;
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (ok)
                    tl[count + __popc(m & lanemask_lt())] =
                        make_uint2((static_cast<uint32_t>(y) << 16) | static_cast<uint32_t>(x), __float_as_uint(iv));
                count += __popc(m);
            }
            gated += static_cast<unsigned>(count);
        } else {
            // Entries per take: enough to keep every warp busy, 32 to kCapQ.
            const int n = qinCount;
            const int warps = gridDim.x * kCasWarps;
            const int chunk = min(kCapQ, max(32, ((n + warps - 1) / warps + 31) & ~31));
            const int64_t base = static_cast<int64_t>(t) * chunk;
            if (base >= n) break;
            count = static_cast<int>(n - base < chunk ? n - base : chunk);
            for (int i = lane; i < count; i += 32) lst[i] = qin[base + i];
        }
        __syncwarp();
        if (tileLevel >= 0) {
            // One level for the whole list: every stump is decoded once for up
            // to 128 windows (4 per lane), whose integral loads are then in
            // flight together.  Each window's sum still adds its stumps in
            // order from 0.0f.
            const CasLevel& L = P.levels[tileLevel];
            const uint32_t* sum = L.sum;
            const int pitch = static_cast<int>(L.pitch);
            for (int si = s0; si < s1 && count > 0; ++si) {
                const DStage st = P.stages[si];
                evals += static_cast<unsigned long long>(count) * static_cast<unsigned>(st.ntrees);
                int nc = 0;
                for (int g0 = 0; g0 < count; g0 += 128) {
                    const int ng = min(4, (count - g0 + 31) >> 5);  // groups of 32 in this block
                    int b[4];
                    float inv[4], acc[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int i = g0 + 32 * q + lane;
                        b[q] = 0;
                        inv[q] = 0.0f;
                        acc[q] = 0.0f;
                        if (q < ng && i < count) {
                            const uint2 e = tl[i];
                            b[q] = static_cast<int>(e.x >> 16) * pitch + static_cast<int>(e.x & 0xFFFFu);
                            inv[q] = __uint_as_float(e.y);
                        }
                    }
                    for (int k = 0; k < st.ntrees; ++k) {
                        LevelStump d;
                        decode_stump(P.stumps + st.first + k, pitch, d);
                        // the stump is the same in every lane: one branch per stump
                        auto eval4 = [&](auto shape) {
                            constexpr int S = decltype(shape)::value;
#pragma unroll
                            for (int q = 0; q < 4; ++q)
                                if (q < ng) acc[q] = __fadd_rn(acc[q], decoded_value_shared<S>(d, sum, b[q], inv[q]));
                        };
                        switch (decoded_sharing(d)) {
                            case 1: eval4(std::integral_constant<int, 1>()); break;
                            case 2: eval4(std::integral_constant<int, 2>()); break;
                            case 3: eval4(std::integral_constant<int, 3>()); break;
                            default: eval4(std::integral_constant<int, 0>()); break;
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (q >= ng) break;
                        const int i = g0 + 32 * q + lane;
                        const bool act = i < count;
                        uint2 e = make_uint2(0u, 0u);
                        if (act) e = tl[i];
                        const bool pass = act && !(acc[q] < st.threshold);
                        const unsigned m = __ballot_sync(0xffffffffu, pass);
                        __syncwarp();
                        if (pass) {
                            if (last && si + 1 == s1) e.y = __float_as_uint(acc[q]);  // the detection's score
                            tl[nc + __popc(m & lanemask_lt())] = e;
                        }
                        nc += __popc(m);
                        __syncwarp();
                    }
                }
                count = nc;
            }
        }
        for (int si = s0; si < s1 && count > 0 && tileLevel < 0; ++si) {
            const DStage st = P.stages[si];
            evals += static_cast<unsigned long long>(count) * static_cast<unsigned>(st.ntrees);
            int nc = 0;
            for (int g = 0; g < count; g += 32) {
                const int i = g + lane;
                const bool act = i < count;
                QEntry e{};
                float s = 0.0f;
                if (act) {
                    e = lst[i];
                    const CasLevel& L = P.levels[e.level];
                    const int64_t Pi = L.pitch;
                    const int64_t b = static_cast<int64_t>(e.xy >> 16) * Pi + static_cast<int64_t>(e.xy & 0xFFFFu);
                    s = stage_sum(P.stumps, st, L.sum, Pi, b, e.inv);
                }
                const bool pass = act && !(s < st.threshold);
                const unsigned m = __ballot_sync(0xffffffffu, pass);
                __syncwarp();
                if (pass) {
                    e.score = s;
                    lst[nc + __popc(m & lanemask_lt())] = e;
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
            if (act) {
                if (tileLevel >= 0) {
                    const uint2 c = tl[i];
                    e.level = static_cast<uint32_t>(tileLevel);
                    e.xy = c.x;
                    if (last)
                        e.score = __uint_as_float(c.y);
                    else
                        e.inv = __uint_as_float(c.y);
                } else {
                    e = lst[i];
                }
            }
            if (last)
                emit_warp(P, e, act);
            else
                push_queue(qout, qoutCount, P.qcap, act, e);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Deep pass: SL windows per warp, 32/SL lanes per window.  Each window slot
// holds the window's (winW+1) x (winH+1) integral patch in shared memory as
// floats; per step every slot evaluates its next 32/SL stumps per lane
// evaluation (lane j of the slot: stumps k0 + j, k0 + j + 32/SL, ...).
//
// A stage is decided from an order-free sum: each lane adds its own leaf
// values, and at the end of the stage a butterfly over the slot's lanes gives
// every lane the same total.  Any way of summing N terms, and the reference's
// sequential FP32 sum from 0.0f, lies within the stage's `tol` of the exact
// sum (tol >= (gamma(N-1) + gamma(N+5)) * sum of max|leaf|, gamma(k) =
// k u / (1 - k u), u = 2^-24), so a total at or above threshold + tol passes
// the reference's test !(acc < threshold) and one below threshold - tol fails
// it.  A slot whose total lies in between, or that passes the last stage
// (whose sum is the detection's score), replays the stage exactly: the values
// go through a per-warp shared buffer and each slot adds them in stump order
// from 0.0f, the reference's sequential FP32 sum.  A slot whose window is
// rejected or accepted takes the next window from the queue; the whole warp
// copies the new window's patch.
//
// Per-warp shared memory: 32 * kDeepEvals floats of values, then SL patches,
// element o of slot s at patches[SL * o + s] (two slots interleaved, so their
// loads fall in different banks: even and odd).  With the stumps of each
// stage reordered by detect.cu spread_banks, the 16 stumps that one load
// instruction of a slot reads mostly have distinct o mod 16, i.e. distinct
// banks; the exact replay puts each value back at the position its stump had
// before the reordering.
// ---------------------------------------------------------------------------
constexpr int kDeepEvals = 3;  // stumps a lane evaluates per step
constexpr int kDeepBlock = 48; // stumps reordered among themselves (a step of 2 slots; half a step of 1)
__host__ __device__ constexpr int deep_warp_floats(int slots, int patchElems) {
    return 32 * kDeepEvals + ((slots * patchElems + 3) & ~3);
}

template <int SL>
__device__ __forceinline__ void deep_pass(const DevPlan& P, float* wsm, const QEntry* q, int n,
                                          unsigned long long* workCounter, unsigned long long& evals) {
    constexpr int LPS = 32 / SL;           // lanes per slot
    constexpr int SPS = LPS * kDeepEvals;  // stumps per slot per step
    static_assert(SPS % kDeepBlock == 0 && LPS % 16 == 0, "steps hold whole reordering blocks of 16-stump groups");
    const int lane = threadIdx.x & 31;
    const int slot = lane / LPS, j = lane % LPS;
    const int pw = P.winW + 1, ph = P.winH + 1;
    float* vals = wsm;  // per slot SPS values in stump order
    float* patches = wsm + 32 * kDeepEvals;
    const float* myPatch = patches + slot;
    const bool spread = P.spreadStumps != 0;
    const uint32_t m0 = spread ? 0x3FFu : 0xFFFFu;
    int qi = -1;  // queue index of the slot's window, -1 = empty
    QEntry e{};
    int si = 0, k0 = 0;
    DStage st{0, 0, 0.0f, 0.0f};  // P.stages[si], read when si changes
    float acc = 0.0f, lacc = 0.0f, score = 0.0f;
    bool exact = false;  // the slot replays its stage with the sequential sum
    bool more = true;
    for (;;) {
        // Refill empty slots one window at a time; all lanes copy the patch.
        while (more) {
            const unsigned empty = __ballot_sync(0xffffffffu, qi < 0 && j == 0);
            if (!empty) break;
            const int s = (__ffs(empty) - 1) / LPS;
            unsigned long long t = 0;
            if (lane == 0) t = atomicAdd(workCounter, 1ull);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= static_cast<unsigned long long>(n)) {
                more = false;
                break;
            }
            const QEntry ne = q[t];
            const CasLevel& L = P.levels[ne.level];
            const uint32_t* sum = L.sum;
            const int64_t Pi = L.pitch;
            const int64_t b = static_cast<int64_t>(ne.xy >> 16) * Pi + static_cast<int64_t>(ne.xy & 0xFFFFu);
            float* dst = patches + s;
            // 8 rows' loads in flight before their stores
            for (int c = lane; c < pw; c += 32)
                for (int r0 = 0; r0 < ph; r0 += 8) {
                    uint32_t v[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (r0 + k < ph) v[k] = sum[b + (r0 + k) * Pi + c];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (r0 + k < ph) dst[SL * ((r0 + k) * pw + c)] = corner_f(v[k]);
                }
            if (slot == s) {
                qi = static_cast<int>(t);
                e = ne;
                si = P.deepFrom;
                st = P.stages[si];
                k0 = 0;
                acc = 0.0f;
                lacc = 0.0f;
                exact = false;
                score = ne.score;
            }
        }
        if (!__any_sync(0xffffffffu, qi >= 0)) break;
        __syncwarp();
        const bool active = qi >= 0;
        float c[kDeepEvals];
#pragma unroll
        for (int ev = 0; ev < kDeepEvals; ++ev) {
            const int k = k0 + ev * LPS + j;
            c[ev] = 0.0f;
            if (active && k < st.ntrees) c[ev] = patch_stump_value<SL>(P.pstumps, st.first + k, myPatch, e.inv, m0);
        }
        const int m = active ? min(SPS, st.ntrees - k0) : 0;
        if (__any_sync(0xffffffffu, exact)) {
#pragma unroll
            for (int ev = 0; ev < kDeepEvals; ++ev) {
                int pos = ev * LPS + j;  // k - k0
                const int k = k0 + pos;
                if (spread && exact && k < st.ntrees)
                    pos = k - k % kDeepBlock - k0 +
                          static_cast<int>((__ldg(&P.pstumps.b[st.first + k].z) >> 10) & 63u);
                vals[slot * SPS + pos] = c[ev];
            }
            __syncwarp();
            if (exact) {
                const float4* v4 = reinterpret_cast<const float4*>(vals + slot * SPS);
#pragma unroll
                for (int g = 0; g < SPS / 4; ++g) {
                    const float4 x = v4[g];
                    if (4 * g + 0 < m) acc = __fadd_rn(acc, x.x);
                    if (4 * g + 1 < m) acc = __fadd_rn(acc, x.y);
                    if (4 * g + 2 < m) acc = __fadd_rn(acc, x.z);
                    if (4 * g + 3 < m) acc = __fadd_rn(acc, x.w);
                }
            }
            __syncwarp();
        }
        if (!exact) {
#pragma unroll
            for (int ev = 0; ev < kDeepEvals; ++ev) lacc = __fadd_rn(lacc, c[ev]);
        }
        if (j == 0) evals += static_cast<unsigned>(m);
        k0 += SPS;
        const bool done = active && k0 >= st.ntrees;
        float tot = lacc;
        if (__any_sync(0xffffffffu, done && !exact)) {
#pragma unroll
            for (int o = LPS / 2; o > 0; o >>= 1) tot = __fadd_rn(tot, __shfl_xor_sync(0xffffffffu, tot, o));
        }
        if (done) {
            // 1 pass, 0 reject, -1 replay the stage exactly
            int outcome;
            if (exact)
                outcome = acc < st.threshold ? 0 : 1;
            else if (tot < __fsub_rd(st.threshold, st.tol))
                outcome = 0;
            else if (tot >= __fadd_ru(st.threshold, st.tol) && si + 1 < P.nStages)
                outcome = 1;
            else
                outcome = -1;
            if (outcome < 0) {
                exact = true;
                k0 = 0;
                acc = 0.0f;
            } else {
                exact = false;
                lacc = 0.0f;
                if (outcome == 0) {
                    qi = -1;
                } else {
                    score = acc;  // exact on the last stage, which is always replayed
                    ++si;
                    k0 = 0;
                    acc = 0.0f;
                    if (si < P.nStages) st = P.stages[si];
                    if (si >= P.nStages) {
                        if (j == 0) {
                            const CasLevel& L = P.levels[e.level];
                            const int slotOut = atomicAdd(P.counts + L.image, 1);
                            if (slotOut < P.detCap)
                                P.dets[static_cast<size_t>(L.image) * P.detCap + slotOut] =
                                    make_detection(L, e, P.winW, P.winH, score);
                        }
                        qi = -1;
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Grouping phases (groupRectangles on the device, see group_dev.cuh), between
// the layout barrier and the output: x histogram, x-order slots, similar
// pairs and unions, cluster sums, best member, clusters, containment and
// cluster order.  Returns 0 when a grid barrier failed, 2 when the grouping
// stopped on an error flag (the host fails the call), 1 when it finished.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned char* dsmem_ptr() {
    extern __shared__ __align__(16) unsigned char dsmem[];
    return dsmem;
}

__device__ __noinline__ int group_phases(const DevPlan& P, GridSync* G, unsigned& epoch, unsigned long long tmo,
                                          int64_t gtid, int64_t gthreads, int64_t gw, int64_t nw, int lane) {
    const GroupPlan& GP = P.grp;
    CtrlHead* C = P.ctrl;
    const int rawTotal = ld_volatile(&C->rawTotal);
    const int keptTotal = ld_volatile(&C->compactTotal);
    auto detAt = [&](int64_t t, int& img) {
        img = image_of(P.rawOff, P.nImg, t);
        return ldl2_det(P.dets + static_cast<size_t>(img) * P.detCap + static_cast<size_t>(t - ldl2(P.rawOff + img)));
    };
    auto keptOf = [&](int img) { return min(min(ldl2(P.counts + img), P.detCap), GP.limit); };

    // a. x histogram of each image's kept detections
    for (int64_t t = gtid; t < rawTotal; t += gthreads) {
        int i;
        const vj_detection d = detAt(t, i);
        if (d.x < 0 || d.x >= GP.histBase[i + 1] - GP.histBase[i]) {
            atomicExch(&C->grpError, 1);  // outside the image: cannot happen for level windows
            continue;
        }
        if (det_key(d) <= ldl2(P.selKey + i)) atomicAdd(GP.hist + GP.histBase[i] + d.x, 1);
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;
    if (ld_volatile(&C->grpError) != 0) return 2;

    // b. per image, exclusive scan of the histogram into slot cursors: a
    // block per image, each thread over a contiguous run of bins
    {
        int* wsum = reinterpret_cast<int*>(dsmem_ptr());
        const int wib = threadIdx.x >> 5;
        for (int i = blockIdx.x; i < P.nImg; i += gridDim.x) {
            int* h = GP.hist + GP.histBase[i];
            const int nb = static_cast<int>(GP.histBase[i + 1] - GP.histBase[i]);
            const int per = (nb + kCasThreads - 1) / kCasThreads;
            const int b0 = min(nb, static_cast<int>(threadIdx.x) * per), b1 = min(nb, b0 + per);
            int sum = 0;
            for (int b = b0; b < b1; ++b) sum += ldl2(h + b);
            int inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += u;
            }
            if (lane == 31) wsum[wib] = inc;
            __syncthreads();
            if (wib == 0) {
                const int v = lane < kCasWarps ? wsum[lane] : 0;
                int wi = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, wi, o);
                    if (lane >= o) wi += u;
                }
                if (lane < kCasWarps) wsum[lane] = wi - v;
            }
            __syncthreads();
            int run = ldl2(P.offsets + i) + wsum[wib] + inc - sum;
            for (int b = b0; b < b1; ++b) {
                const int v = ldl2(h + b);
                h[b] = run;
                run += v;
            }
            __syncthreads();
        }
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // c. kept detections into x order (the order among equal x is free: the
    // pair search below covers every pair within the x reach either way)
    for (int64_t t = gtid; t < rawTotal; t += gthreads) {
        int i;
        const vj_detection d = detAt(t, i);
        const unsigned long long key = det_key(d);
        if (key > ldl2(P.selKey + i) || d.x < 0 || d.x >= GP.histBase[i + 1] - GP.histBase[i]) continue;
        const int sl = atomicAdd(GP.hist + GP.histBase[i] + d.x, 1);
        GP.x[sl] = d.x;
        GP.y[sl] = d.y;
        GP.w[sl] = d.w;
        GP.h[sl] = d.h;
        GP.score[sl] = d.score;
        GP.key[sl] = key;
        GP.parent[sl] = sl;
        GP.image[sl] = i;
        GP.cnt[sl] = 0;
        GP.best[sl] = 0u;
        GP.sumX[sl] = 0ull;
        GP.sumY[sl] = 0ull;
        GP.sumW[sl] = 0ull;
        GP.sumH[sl] = 0ull;
        GP.bestKey[sl] = ~0ull;
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // d. similar pairs (similarRects, face_vision_engine.cu:585-616) within
    // the x reach of the earlier rectangle, joined as found: a warp per RG
    // consecutive rectangles (RG = the rectangles per warp, 1 to 32), whose
    // lanes first load one rectangle each (its box and the end of its
    // image's range); then, rectangle by rectangle, the lanes go over the
    // later rectangles 32 at a time (x order ends the scan at the first chunk
    // that reaches past the reach)
    const int RG = static_cast<int>(min(static_cast<int64_t>(32), max(static_cast<int64_t>(1), keptTotal / nw)));
    for (int64_t p0 = gw * RG; p0 < keptTotal; p0 += nw * RG) {
        const int64_t pl = p0 + lane;
        int lend = 0, lx = 0, ly = 0, lw = 0, lh = 0;
        if (lane < RG && pl < keptTotal) {
            const int li = ldl2(GP.image + pl);
            lend = ldl2(P.offsets + li) + keptOf(li);
            lx = ldl2(GP.x + pl), ly = ldl2(GP.y + pl), lw = ldl2(GP.w + pl), lh = ldl2(GP.h + pl);
        }
        const int rn = static_cast<int>(min(static_cast<int64_t>(RG), keptTotal - p0));
        for (int r = 0; r < rn; ++r) {
            const int64_t p = p0 + r;
            const int end = __shfl_sync(0xffffffffu, lend, r);
            const int ax = __shfl_sync(0xffffffffu, lx, r), ay = __shfl_sync(0xffffffffu, ly, r);
            const int aw = __shfl_sync(0xffffffffu, lw, r), ah = __shfl_sync(0xffffffffu, lh, r);
            const int reach = __float2int_rz(__fmul_rn(__fmul_rn(GP.eps, static_cast<float>(aw + ah)), 0.5f));
            // two chunks per step, both loaded before either is tested; once
            // a chunk holds a rectangle past the reach, every later one is
            // past it too (x order), so the pairs found are the same
            for (int q0 = static_cast<int>(p) + 1; q0 < end; q0 += 64) {
                int bx[2], by[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int q = q0 + 32 * h + lane;
                    bx[h] = q < end ? ldl2(GP.x + q) : INT_MAX;
                    by[h] = q < end ? ldl2(GP.y + q) : 0;
                }
                bool anyPast = false;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int q = q0 + 32 * h + lane;
                    const bool past = q >= end || bx[h] > ax + reach;
                    bool sim = false;
                    if (!past && abs(ay - by[h]) <= reach) {
                        const int bw = ldl2(GP.w + q), bh = ldl2(GP.h + q);
                        const int delta = __float2int_rz(
                            __fmul_rn(__fmul_rn(GP.eps, static_cast<float>(min(aw, bw) + min(ah, bh))), 0.5f));
                        sim = abs(ax - bx[h]) <= delta && abs(ay - by[h]) <= delta &&
                              abs(ax + aw - bx[h] - bw) <= delta && abs(ay + ah - by[h] - bh) <= delta;
                    }
                    if (sim && !gf_unite(GP.parent, GP.key, static_cast<int>(p), q)) atomicExch(&C->grpError, 1);
                    anyPast |= past;
                }
                if (__any_sync(0xffffffffu, anyPast)) break;
            }
        }
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // e. roots, sizes, sums and the largest score of each cluster (the root
    // goes to its own array: parent entries can still be rewritten to other
    // ancestors by concurrent finds)
    for (int64_t p = gtid; p < keptTotal; p += gthreads) {
        const int r = gf_find(GP.parent, static_cast<int>(p));
        GP.root[p] = r;
        atomicAdd(GP.cnt + r, 1);
        atomicAdd(GP.sumX + r, static_cast<unsigned long long>(ldl2(GP.x + p)));
        atomicAdd(GP.sumY + r, static_cast<unsigned long long>(ldl2(GP.y + p)));
        atomicAdd(GP.sumW + r, static_cast<unsigned long long>(ldl2(GP.w + p)));
        atomicAdd(GP.sumH + r, static_cast<unsigned long long>(ldl2(GP.h + p)));
        atomicMax(GP.best + r, score_order(ldl2(GP.score + p)));
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // f. the first member (canonical order) among those with the largest score
    for (int64_t p = gtid; p < keptTotal; p += gthreads) {
        const int r = ldl2(GP.root + p);
        if (score_order(ldl2(GP.score + p)) == ldl2(GP.best + r)) atomicMin(GP.bestKey + r, ldl2(GP.key + p));
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // g. clusters with more than minN members, written by their best member
    for (int64_t p = gtid; p < keptTotal; p += gthreads) {
        const int r = ldl2(GP.root + p);
        const int n = ldl2(GP.cnt + r);
        const unsigned long long key = ldl2(GP.key + p);
        if (key != ldl2(GP.bestKey + r) || n <= GP.minN) continue;
        const int i = ldl2(GP.image + p);
        const int c = atomicAdd(P.ccount + i, 1);
        GCluster g;
        const unsigned long long un = static_cast<unsigned long long>(n);
        g.x = static_cast<int>(ldl2(GP.sumX + r) / un);
        g.y = static_cast<int>(ldl2(GP.sumY + r) / un);
        g.w = static_cast<int>(ldl2(GP.sumW + r) / un);
        g.h = static_cast<int>(ldl2(GP.sumH + r) / un);
        g.n = n;
        g.scaleIdx = static_cast<int>(key >> 32);
        g.score = ldl2(GP.score + p);
        g.image = i;
        g.key = ldl2(GP.key + r);
        GP.cl[ldl2(P.offsets + i) + c] = g;
        // the cluster's slot into the list phase h walks (parent, whose
        // entries no phase after e reads)
        GP.parent[atomicAdd(&C->clTotal, 1)] = ldl2(P.offsets + i) + c;
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;

    // h. containment filter against every other cluster of the image, and
    // each cluster's rank by first-member key: a warp per listed cluster
    const int clTotal = ld_volatile(&C->clTotal);
    for (int64_t t = gw; t < clTotal; t += nw) {
        const int slot = ldl2(GP.parent + t);
        const GCluster a = ldl2_cluster(GP.cl + slot);
        const int off = ldl2(P.offsets + a.image), cc = ldl2(P.ccount + a.image);
        const int k = slot - off;
        int rank = 0;
        bool drop = false;
        for (int j = lane; j < cc; j += 32) {
            const GCluster b = ldl2_cluster(GP.cl + off + j);
            rank += b.key < a.key ? 1 : 0;
            if (j == k) continue;
            const int dx = __float2int_rz(__fmul_rn(static_cast<float>(b.w), GP.eps));
            const int dy = __float2int_rz(__fmul_rn(static_cast<float>(b.h), GP.eps));
            if (a.x >= b.x - dx && a.y >= b.y - dy && a.x + a.w <= b.x + b.w + dx && a.y + a.h <= b.y + b.h + dy &&
                (b.n > max(3, a.n) || a.n < 3))
                drop = true;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rank += __shfl_xor_sync(0xffffffffu, rank, o);
        drop = __any_sync(0xffffffffu, drop);
        if (lane == 0) GP.order[off + rank] = drop ? -1 - k : k;
    }
    if (!grid_barrier(G, epoch, tmo)) return 0;
    return ld_volatile(&C->grpError) != 0 ? 2 : 1;
}

// ---------------------------------------------------------------------------
// The persistent detection kernel: every phase of a batch in one cooperative
// launch, phases separated by grid barriers.
//   1. pyramid: resize chain positions 0, 1, ... (level k from level k-1);
//   2. integral images of every level: row pass, then one column walk per
//      32-column chunk (large batches) or column totals and a column scan;
//   3. tile pass (lane-per-window) over every level of every image;
//   4. lane-per-window queue passes (optional);
//   5. warp-per-window deep pass over the remaining stages;
//   6. layout of each image's kept raw detections (truncation key per image);
//   7. with grouping, groupRectangles (group_phases);
//   8. output: each image's clusters in order, or its raw detections, into
//      the host-mapped buffer.
// ---------------------------------------------------------------------------
template <int TH, int MINB, int SL>
__global__ void __launch_bounds__(kCasThreads, MINB)
detect_persistent_kernel(const DevPlan* __restrict__ plan) {
    extern __shared__ __align__(16) unsigned char dsmem[];
    const DevPlan& P = *plan;
    CtrlHead* C = P.ctrl;
    GridSync* G = &C->sync;
    unsigned epoch = 0;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const bool stamper = blockIdx.x == 0 && threadIdx.x == 0;
    const unsigned long long tmo = P.barrierTimeoutNs ? P.barrierTimeoutNs : kBarrierTimeoutNs;
    if (stamper) G->stamp[0] = global_ns();
    if (P.holdBlock >= 0 && blockIdx.x == static_cast<unsigned>(P.holdBlock)) return;
    const int64_t gtid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t gthreads = static_cast<int64_t>(gridDim.x) * blockDim.x;
    if (P.grp.enabled)
        for (int64_t t = gtid; t < P.grp.histTotal; t += gthreads) P.grp.hist[t] = 0;

    // 1. pyramid
    for (int p = 0; p < P.nResize; ++p) {
        const int j0 = P.rjFirst[p], j1 = P.rjFirst[p + 1];
        const int64_t items = P.rjItems[p];
        for (int64_t it = gw; it < items; it += nw) resize_item(P.rjobs + j0, j1 - j0, it, lane);
        if (!grid_barrier(G, epoch, tmo)) return;
    }
    if (stamper) G->stamp[1] = global_ns();

    // 2. integral images
    for (int64_t r = gw; r < P.ip.rows; r += nw) ii_row_item(P.iijobs, P.nLevels, r, lane);
    if (!grid_barrier(G, epoch, tmo)) return;
    if (P.colWalk) {
        for (int64_t it = gw; it < P.ip.walkItems; it += nw) ii_col_walk_item(P.iijobs, P.nLevels, it, lane);
    } else {
        for (int64_t it = gw; it < P.ip.items; it += nw)
            ii_col_total_item(P.iijobs, P.nLevels, it, lane, P.ip.totPitch, P.totS, P.totQ);
        if (!grid_barrier(G, epoch, tmo)) return;
        for (int64_t it = gw; it < P.ip.items; it += nw)
            ii_col_scan_item(P.iijobs, P.nLevels, it, lane, P.ip.totPitch, P.totS, P.totQ);
    }
    if (!grid_barrier(G, epoch, tmo)) return;
    if (stamper) G->stamp[2] = global_ns();

    unsigned long long gated = 0, evals = 0, deepEvals = 0;
    QEntry* lst = reinterpret_cast<QEntry*>(dsmem) + static_cast<size_t>(wib) * 16 * TH;  // 32 * TH * 8 bytes

    // 3. tile pass -> queue 0 (or detections)
    lane_pass<TH>(P, lst, nullptr, 0, 0, P.tileStages, &C->work[0], P.q[0], &C->qcount[0], gated, evals);
    if (!grid_barrier(G, epoch, tmo)) return;
    if (stamper) G->stamp[3] = global_ns();

    // 4. queue passes: queue m -> queue m+1
    for (int m = 0; m < P.nQueuePasses; ++m) {
        const int s0 = m == 0 ? P.tileStages : P.queueEnd[m - 1];
        const int nIn = min(C->qcount[m], P.qcap);
        lane_pass<TH>(P, lst, P.q[m & 1], nIn, s0, P.queueEnd[m], &C->work[1 + m], P.q[(m + 1) & 1],
                      &C->qcount[m + 1], gated, evals);
        if (!grid_barrier(G, epoch, tmo)) return;
    }
    if (stamper) G->stamp[4] = global_ns();

    // 5. deep pass
    if (P.deepFrom < P.nStages) {
        const int m = P.nQueuePasses;
        const int nIn = min(C->qcount[m], P.qcap);
        float* wsm = reinterpret_cast<float*>(dsmem) +
                     static_cast<size_t>(wib) * deep_warp_floats(SL, (P.winW + 1) * (P.winH + 1));
        deep_pass<SL>(P, wsm, P.q[m & 1], nIn, &C->work[kQueues], deepEvals);
    }
    // lane passes count the same totals in every lane; the deep pass counts
    // per slot in the slot's first lane
    unsigned long long deepSum = deepEvals;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) deepSum += __shfl_xor_sync(0xffffffffu, deepSum, o);
    if (lane == 0) {
        if (gated) atomicAdd(&C->stats[0], gated);
        if (evals + deepSum) atomicAdd(&C->stats[1], evals + deepSum);
    }
    if (!grid_barrier(G, epoch, tmo)) return;
    if (stamper) G->stamp[5] = global_ns();

    // 6. layout: block 0 places each image's kept raw detections (offsets:
    // min(count, detCap), and with grouping at most `limit` of them) and its
    // raw detections in flat order (rawOff); with grouping every block then
    // finds the truncation key of its images.
    const GroupPlan& GP = P.grp;
    const bool grp = GP.enabled != 0;
    if (blockIdx.x == 0) {
        int* part = reinterpret_cast<int*>(dsmem);
        const int n = P.nImg;
        const int per = (n + kCasThreads - 1) / kCasThreads;
        const int i0 = min(n, static_cast<int>(threadIdx.x) * per), i1 = min(n, i0 + per);
        int s = 0, sr = 0;
        for (int i = i0; i < i1; ++i) {
            const int raw = min(ldl2(P.counts + i), P.detCap);
            sr += raw;
            s += grp ? min(raw, GP.limit) : raw;
        }
        part[threadIdx.x] = s;
        part[kCasThreads + threadIdx.x] = sr;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0, runr = 0;
            for (int k = 0; k < kCasThreads; ++k) {
                const int v = part[k], vr = part[kCasThreads + k];
                part[k] = run;
                part[kCasThreads + k] = runr;
                run += v;
                runr += vr;
            }
            C->compactTotal = run;
            C->compactOverflow = run > P.hostCap ? 1 : 0;
            C->rawTotal = runr;
            C->grpOverflow = grp && run > GP.cap ? 1 : 0;
        }
        __syncthreads();
        int off = part[threadIdx.x], offr = part[kCasThreads + threadIdx.x];
        for (int i = i0; i < i1; ++i) {
            const int raw = min(ldl2(P.counts + i), P.detCap);
            P.offsets[i] = off;
            P.rawOff[i] = offr;
            off += grp ? min(raw, GP.limit) : raw;
            offr += raw;
        }
        __syncthreads();
    }
    if (grp)
        for (int i = blockIdx.x; i < P.nImg; i += gridDim.x) {
            const int raw = min(ldl2(P.counts + i), P.detCap);
            if (raw > GP.limit) {
                const unsigned long long k = block_select_key(P.dets + static_cast<size_t>(i) * P.detCap, raw,
                                                              GP.limit, reinterpret_cast<unsigned*>(dsmem));
                if (threadIdx.x == 0) P.selKey[i] = k;
            } else if (threadIdx.x == 0) {
                P.selKey[i] = ~0ull;
            }
        }
    if (!grid_barrier(G, epoch, tmo)) return;
    bool doGroup = grp && ld_volatile(&C->grpOverflow) == 0 && ld_volatile(&C->compactOverflow) == 0;
    if (doGroup) {
        const int r = group_phases(P, G, epoch, tmo, gtid, gthreads, gw, nw, lane);
        if (r == 0) return;
        doGroup = r == 1;
    }
    if (stamper) G->stamp[6] = global_ns();

    // 7. output into the host-mapped buffer: the grouped detections of each
    // image in cluster order, or its raw detections.
    if (doGroup) {
        for (int64_t i = gw; i < P.nImg; i += nw) {
            const int off = ldl2(P.offsets + i), cc = ldl2(P.ccount + i);
            int outN = 0;
            for (int b = 0; b < cc; b += 32) {
                const int k = b + lane;
                const int v = k < cc ? ldl2(GP.order + off + k) : -1;
                const bool keep = v >= 0;
                const unsigned m = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const GCluster c = ldl2_cluster(GP.cl + off + v);
                    vj_detection d;
                    d.x = c.x;
                    d.y = c.y;
                    d.w = c.w;
                    d.h = c.h;
                    d.scaleIdx = c.scaleIdx;
                    d.score = c.score;
                    P.hostDets[off + outN + __popc(m & lanemask_lt())] = d;
                }
                outN += __popc(m);
            }
            if (lane == 0) P.gcount[i] = outN;
        }
    } else if (!grp && C->compactOverflow == 0) {
        for (int64_t i = gw; i < P.nImg; i += nw) {
            const int cnt = min(ldl2(P.counts + i), P.detCap);
            const int off = ldl2(P.offsets + i);
            const vj_detection* src = P.dets + static_cast<size_t>(i) * P.detCap;
            for (int k = lane; k < cnt; k += 32) P.hostDets[off + k] = ldl2_det(src + k);
        }
    }
    if (stamper) G->stamp[7] = global_ns();
}

}  // namespace vjgb
