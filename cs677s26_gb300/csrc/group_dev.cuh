// Device side of groupRectangles (face_vision_engine.cu:1401-1539): the
// phases the persistent detection kernel runs after its deep pass, so that a
// grouped call hands the host finished clusters.
//
// The reference's result is a function of the similar-pair graph, not of the
// order its sweep visits pairs in:
//   - the clusters are the connected components of "similarRects" pairs (a
//     pair is found by the sweep from whichever rectangle comes first in x
//     order, because delta(a, b) <= reach(a)), so a lock-free union-find over
//     every similar pair gives the same components;
//   - a cluster's averages are int64 sums divided by its size;
//   - its score and scaleIdx are those of the first member, in input order,
//     with the largest score (strict '>' over the input), and the input is
//     the canonical (scaleIdx, y, x) order, so the key of that member is the
//     smallest canonical key among the members whose score equals the
//     maximum (+0.0 and -0.0 compare equal, as in the reference);
//   - the containment filter compares every kept cluster with every other.
// Only the order of the output clusters is not fixed by the reference (its
// raw detections arrive in atomic order); here clusters come out by the
// canonical key of their first member.
//
// The union-find hooks a root under the root with the smaller canonical key
// (keys are unique within an image), so parent chains strictly decrease in
// key and every component ends with its first member as root.
#pragma once

#include <cstdint>

#include "common.h"

namespace vjgb {

struct GCluster {
    int x, y, w, h;
    int n, scaleIdx;
    float score;
    int image;
    unsigned long long key;  // canonical key of the cluster's first member
};
static_assert(sizeof(GCluster) == 40, "GCluster is 40 bytes");

// Arrays of the grouping phases, `cap` slots each; slot s of image i is
// offsets[i] + k for its k-th kept raw detection in x order.
struct GroupPlan {
    int enabled;   // 1: group on the device
    int minN;      // max(1, minNeighbors)
    int limit;     // raw detections kept per image, first in canonical order
    int cap;       // slots of the arrays below
    float eps;
    int pad;
    const int64_t* histBase;  // nImg + 1 bin offsets into hist (image i: w_i + 1 bins)
    int* hist;                // zeroed at the start of the launch
    int64_t histTotal;
    int *x, *y, *w, *h;
    float* score;
    unsigned long long* key;
    int* parent;
    int* root;   // root of each slot, written once after the unions
    int* image;
    int* cnt;
    unsigned* best;
    unsigned long long *sumX, *sumY, *sumW, *sumH;
    unsigned long long* bestKey;
    GCluster* cl;
    int* order;
};

// Bytes of the grouping arrays per slot, split over the two queue buffers
// they reuse: [x y w h score parent root image | key] and
// [cnt best order | sums bestKey | clusters].
constexpr int64_t kGroupBytesA = 8 * 4 + 8;
constexpr int64_t kGroupBytesB = 3 * 4 + 5 * 8 + sizeof(GCluster);

// The canonical key of a detection: the host's canonical sort key.
__host__ __device__ __forceinline__ unsigned long long det_key(const vj_detection& d) {
    return (static_cast<unsigned long long>(static_cast<uint32_t>(d.scaleIdx)) << 32) |
           (static_cast<unsigned long long>(static_cast<uint16_t>(d.y)) << 16) |
           static_cast<unsigned long long>(static_cast<uint16_t>(d.x));
}

// Float order as unsigned, with -0.0 and +0.0 equal.
__device__ __forceinline__ unsigned score_order(float f) {
    unsigned b = __float_as_uint(f);
    if ((b & 0x7FFFFFFFu) == 0u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Loads of data other blocks wrote earlier in the same launch go to L2
// (ld.global.cg), so no SM can see a line it cached before the writes.
template <class T>
__device__ __forceinline__ T ldl2(const T* p) {
    return __ldcg(p);
}

__device__ __forceinline__ vj_detection ldl2_det(const vj_detection* p) {
    const int2* q = reinterpret_cast<const int2*>(p);  // records are 8-byte aligned
    const int2 a = __ldcg(q), b = __ldcg(q + 1), c = __ldcg(q + 2);
    vj_detection d;
    d.x = a.x;
    d.y = a.y;
    d.w = b.x;
    d.h = b.y;
    d.scaleIdx = c.x;
    d.score = __int_as_float(c.y);
    return d;
}

__device__ __forceinline__ GCluster ldl2_cluster(const GCluster* p) {
    const int2* q = reinterpret_cast<const int2*>(p);  // records are 8-byte aligned
    const int2 a = __ldcg(q), b = __ldcg(q + 1), c = __ldcg(q + 2), d = __ldcg(q + 3);
    GCluster g;
    g.x = a.x;
    g.y = a.y;
    g.w = b.x;
    g.h = b.y;
    g.n = c.x;
    g.scaleIdx = c.y;
    g.score = __int_as_float(d.x);
    g.image = d.y;
    g.key = __ldcg(reinterpret_cast<const unsigned long long*>(p) + 4);
    return g;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

constexpr int kFindMaxSteps = 1 << 26;
constexpr int kUniteMaxTries = 1 << 24;

// Root of x; halves the path on the way (every write points a node at one of
// its ancestors, which stays valid while other threads hook roots).
__device__ __forceinline__ int gf_find(int* par, int x) {
    int p = ld_volatile(par + x);
    for (int it = 0; p != x && it < kFindMaxSteps; ++it) {
        const int g = ld_volatile(par + p);
        if (g != p) *reinterpret_cast<volatile int*>(par + x) = g;
        x = p;
        p = g;
    }
    return x;
}

// Joins the components of a and b; false only if the retry bound ran out.
__device__ __forceinline__ bool gf_unite(int* par, const unsigned long long* key, int a, int b) {
    for (int t = 0; t < kUniteMaxTries; ++t) {
        a = gf_find(par, a);
        b = gf_find(par, b);
        if (a == b) return true;
        if (__ldcg(key + a) < __ldcg(key + b)) {
            const int s = a;
            a = b;
            b = s;
        }
        if (atomicCAS(par + a, a, b) == a) return true;
    }
    return false;
}

// The k-th smallest canonical key (k >= 1) of n detections, by one block:
// an 8-bit radix select from the top digit.  `sm` holds 256 + 4 words.
__device__ __forceinline__ unsigned long long block_select_key(const vj_detection* d, int n, int k,
                                                               unsigned* sm) {
    unsigned* hist = sm;
    unsigned long long* pre = reinterpret_cast<unsigned long long*>(sm + 256);
    int* rem = reinterpret_cast<int*>(sm + 258);
    if (threadIdx.x == 0) {
        *pre = 0ull;
        *rem = k;
    }
    unsigned long long mask = 0ull;
    for (int dg = 7; dg >= 0; --dg) {
        __syncthreads();
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0u;
        __syncthreads();
        const unsigned long long prefix = *pre;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const unsigned long long key = det_key(ldl2_det(d + j));
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> (8 * dg)) & 0xFFu], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int r = *rem, b = 0;
            while (b < 255 && static_cast<int>(hist[b]) < r) r -= static_cast<int>(hist[b++]);
            *rem = r;
            *pre = prefix | (static_cast<unsigned long long>(b) << (8 * dg));
        }
        mask |= 0xFFull << (8 * dg);
    }
    __syncthreads();
    const unsigned long long out = *pre;
    __syncthreads();
    return out;
}

// Image of flat index t given the exclusive prefix off[0..n-1].
__device__ __forceinline__ int image_of(const int* off, int n, int64_t t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ldl2(off + mid) <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace vjgb
