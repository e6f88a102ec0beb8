// AdaBoost best-weak (decision stump) search and round update on sm_103a.
//
// Reference path (hengyizhu/CS677s26): per round, a tile loop of
// EvaluateFeatureResponsesKernel -> cub::DeviceSegmentedRadixSort ->
// EvaluateAndFindThresholdKernel -> SelectBestInTileKernel
// (src/boosting_core.cu:221-456, src/main.cu:2013-2053), then
// ReduceTileBestCandidatesKernel and the update kernels (main.cu:829-1028).
// Its CPU twin runCpuWeakSearch (main.cu:587-682) defines the pick this file
// reproduces bit for bit.
//
// Design here:
//   1. eval_sort_kernel: one CTA per feature evaluates the exact normalised
//      responses of all samples into shared memory and sorts them with an
//      on-chip stable LSD radix sort (4 x 8-bit digits, ranks from warp
//      ballots, per-warp digit counters).  It writes the sorted sample order (2 B per
//      feature-sample: the sample index, or for up to kTwoCopyMax samples the
//      shared-memory slot of one of two weight copies, chosen against bank
//      conflicts in the sweep) and a bitmask of valid split positions
//      (v[k] + 1e-7f < v[k+1], boosting_core.cu:400).
//   2. sweep_kernel: one warp per feature streams that order, gathers signed
//      weights from shared memory and forms FP32 prefix sums (each lane a run
//      of the feature's sorted positions, 16 at a time with a Kahan-compensated
//      carry, one warp shuffle scan per feature) to
//      get each feature's minimum weighted error to within a proven bound.
//   3. Candidates: every feature whose error is within 2*(bound of the
//      reference's sequential FP32 arithmetic + bound of step 2) of the
//      minimum.  The reference's pick is provably among them.
//   4. refine_kernel: one warp per candidate replays the reference's
//      sequential FP32 totals and sweep exactly (main.cu:626-678): the warp
//      stages each 256-position chunk's weights in sorted order, one lane
//      runs the sequential FP32 chain, all lanes score the valid splits; the
//      winner is the smallest FP32 error, ties to the lower featureIdx.
// With vj_trainer_prepare_stage the orders of step 1 stay resident in HBM for
// all rounds of a stage (the responses do not change within a stage, only
// the weights), so a round costs steps 2-4 only.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "device_util.cuh"

namespace vjgb {
namespace {

constexpr int kSortThreads = 1024;
constexpr int kCntStride = 33;  // per-digit row of 32 warp counters, padded against bank conflicts
constexpr int kSweepThreads = 512;
constexpr int kSmemWeightsMax = 49152;  // samples whose weights fit in shared memory
constexpr int kRefineThreads = 256;
constexpr int kRefineWarps = kRefineThreads / 32;
constexpr float kU = 5.9604645e-08f;    // 2^-24, unit roundoff of FP32

// Stage gate (vj_trainer_set_stage_gate): a device word that the round
// kernels read first; once nonzero, every later round kernel returns at once.
// The round update closes it with 2 when the search found no valid stump, the
// calibration with 1 when the stage meets its targets, so a host can queue a
// stage's rounds without reading anything back between them.
// prmt.b32 whose selector nibbles have bit 3 set: each result byte is the
// top bit of the selected source byte, replicated over the byte.
__device__ __forceinline__ uint32_t prmt_sign(uint32_t a, uint32_t sel) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(0u), "r"(sel));
    return r;
}

__device__ __forceinline__ bool gate_closed(const int* g) {
    return g != nullptr && *reinterpret_cast<const volatile int*>(g) != 0;
}

// Resident stage orders (one row per feature) are stored by lane runs: the
// sweep's lane l owns the L consecutive sorted positions [l*L, (l+1)*L), with
// L = lane_run(n) = ceil(n / 32) rounded up to 16, and step t of a row (256
// slots) holds positions l*L + 8t .. l*L + 8t + 7 of every lane l at slots
// 256t + 8l .. 256t + 8l + 7.  Each 16-byte load of a lane is thus contiguous
// across the warp (512 B per load instruction), and any 8 positions starting
// at a multiple of 8 stay contiguous.  Rows are 32*L positions; positions from
// n up to the next multiple of 8 hold the zero-weight slot (zero_slot).  The
// split bitmask is stored the same way: 16-bit word 32*t + l holds the bits of
// positions l*L + 16t .. l*L + 16t + 15.
__host__ __device__ __forceinline__ int lane_run(int n) { return (((n + 31) / 32) + 15) & ~15; }
// (positions and slots are below 32 * 1024, so 32-bit arithmetic is exact)
__host__ __device__ __forceinline__ int ord_slot(int k, int L) {
    const int l = k / L, r = k - l * L;
    return (r >> 3) * 256 + l * 8 + (r & 7);
}
__host__ __device__ __forceinline__ int gap_word(int k, int L) {
    const int l = k / L, r = k - l * L;
    return (r >> 4) * 32 + l;
}

// Two copies of the round's signed weights in shared memory (n <= kTwoCopyMax):
// copy 0 at [0, n), copy 1 at base + copy1_offset(i) with base = n rounded up
// to 32, where sample i keeps its row of 32 but its column is rotated by
// 7 x row, so the two copies of a sample usually sit in different banks.
// The sort then stores in each resident order slot not the sample index but
// the shared-memory word to read (copy 0: the index itself; copy 1: base +
// copy1_offset), choosing the copy so that the 32 positions one sweep gather
// instruction reads spread over the banks (greedy two-choice assignment:
// about 2.25 wavefronts per gather instead of 3.5 for one copy).  The sums
// are unchanged: every position still adds its own sample's weight.
constexpr int kTwoCopyMax = 24576;
__host__ __device__ __forceinline__ int two_copy_base(int n) { return (n + 31) & ~31; }
__host__ __device__ __forceinline__ uint32_t copy1_offset(uint32_t i) {
    return (i & ~31u) | ((i + 7u * (i >> 5)) & 31u);
}
__host__ __device__ __forceinline__ uint32_t copy1_sample(uint32_t r) {
    return (r & ~31u) | ((r - 7u * (r >> 5)) & 31u);
}
// Shared-memory word that holds +0.0f, after the weights: the slot of the
// padding positions, so a lane past n adds nothing and needs no mask.
__host__ __device__ __forceinline__ int zero_slot(int n, int slotBase) { return slotBase > 0 ? 2 * slotBase : n; }
// Sample index of a resident order slot value.
__host__ __device__ __forceinline__ uint32_t slot_sample(uint32_t v, int slotBase) {
    return (slotBase > 0 && v >= static_cast<uint32_t>(slotBase)) ? copy1_sample(v - slotBase) : v;
}
// Fills a block's shared weights: one copy, or both copies when slotBase > 0,
// and the zero slot.
__device__ __forceinline__ void fill_weights(float* dst, const float* __restrict__ src, int n, int slotBase) {
    // eight loads in flight per thread
    for (int i0 = threadIdx.x; i0 < n; i0 += 8 * blockDim.x) {
        float w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = i0 + u * static_cast<int>(blockDim.x);
            w[u] = i < n ? __ldg(src + i) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = i0 + u * static_cast<int>(blockDim.x);
            if (i < n) {
                dst[i] = w[u];
                if (slotBase > 0) dst[slotBase + copy1_offset(i)] = w[u];
            }
        }
    }
    if (threadIdx.x == 0) dst[zero_slot(n, slotBase)] = 0.0f;
}

struct RoundParams {
    float tp, tn, w;             // active positive / negative weight and their sum
    float window;                // candidate window above the fast minimum
    unsigned int fastMinBits;    // min fast error over features (float bits, >= 0)
    int ncand;                   // number of candidates
    unsigned long long winner;   // (FP32 error bits << 32) | featureIdx; min wins
    int np, nn;                  // active positive / negative sample counts
    int status;                  // 0 ok, 1 no valid split anywhere
    float bfast;                 // bound of |fast error - exact error| (rounded up)
    float lbScale;               // factor taking last round's bounds to this round's weights
    int pruneOK;                 // 1: the bounds hold for this round's weights
    unsigned int nextFeat;       // feature counter of the sweep's work distribution
    int swept;                   // features the sweep streamed this round
};

// Bounds that let the sweep skip features (see sweep_kernel).  Within a
// stage, one AdaBoost update multiplies every active weight by 1 or F and
// divides it by Z, so a feature's exact best error after the update is at
// least min(1, F) / Z times its error before; `scale` is that factor of the
// last update (rounded down, with room for the FP32 rounding of the new
// weights), and `valid` says whether the per-feature bounds and the weight
// shadow describe the current weights.
struct PruneState {
    double F;      // exp(C) of the last update
    float scale;   // min(1, F) / Z * (1 - 4u), at most 1
    int valid;
};

// Mask of the lanes of the warp whose 8-bit digit equals this lane's, from 8
// ballots (one per digit bit): the lanes whose digit differs in some bit are
// the ballot XOR the lane's own bit as an all-ones or all-zero mask.  Byte k
// of lo (hi) has bit k (4 + k) of the digit as its top bit (the four shifted
// copies of the nibble occupy disjoint bits), and prmt_sign spreads that bit
// over the word.
__device__ __forceinline__ uint32_t digit_peers(uint32_t d) {
    uint32_t differ = 0;
    const uint32_t lo = (d & 0xFu) * 0x10204080u, hi = (d >> 4) * 0x10204080u;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const uint32_t own = prmt_sign(b < 4 ? lo : hi, (8u + (b & 3)) * 0x1111u);
        const uint32_t m = __ballot_sync(0xffffffffu, own != 0u);
        differ |= m ^ own;
    }
    return ~differ;
}

// Exclusive scan, in place, of the 256 x 32 per-(digit, warp) counters in
// (digit, warp) order; 1024 threads, thread t scans 8 counters of digit t / 4.
__device__ __forceinline__ void scan_digit_counters(uint32_t* cnt, uint32_t* warpTot) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int d = tid >> 2, w0 = (tid & 3) * 8;
    uint32_t v[8];
    uint32_t run = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t t = cnt[d * kCntStride + w0 + i];
        v[i] = run;
        run += t;
    }
    uint32_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = warpTot[lane];
        uint32_t s = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warpTot[lane] = s - t;
    }
    __syncthreads();
    const uint32_t base = warpTot[warp] + incl - run;
#pragma unroll
    for (int i = 0; i < 8; ++i) cnt[d * kCntStride + w0 + i] = base + v[i];
}

// ---------------------------------------------------------------------------
// 1. Evaluate + on-chip stable radix sort of one feature per CTA.
// ---------------------------------------------------------------------------
// Up to 24 items per thread the sort ping-pongs two index buffers in shared
// memory, so an item's sample index is re-read from the source buffer when it
// is scattered and only its 16-bit rank and 8-bit digit stay in registers;
// 32 items per thread keep the indices in registers (one buffer).
template <int R>
__host__ __device__ constexpr bool sort_ping_pong() { return R <= 24; }

template <int R>
constexpr size_t sort_smem_bytes() {
    return static_cast<size_t>(1024 * R) * (4 + (sort_ping_pong<R>() ? 4 : 2)) + 256 * kCntStride * 4;
}

// Outputs of one sorted feature (every thread of the 1024-thread CTA calls
// this after the last pass): the split bitmask from the sorted keys (keys[]
// in sample order, idx[] the sorted sample order, 16-byte aligned; gnat is
// scratch for n/16 16-bit words), the two-copy slot assignment, and the order
// row, in the lane-run layout when ordPadded.  idx[] is rewritten in place
// (slots, padding).
__device__ __forceinline__ void sort_epilogue(const uint32_t* keys, uint16_t* idx, uint32_t* gnat, int n, int fl,
                                              uint16_t* __restrict__ ordOut, int64_t ordStride, bool ordPadded,
                                              uint16_t* __restrict__ gapOut, int64_t gapStride, int slotBase, int L,
                                              uint16_t* stage = nullptr, int stageCap = 0) {
    const int tid = threadIdx.x;
    // Valid split positions: v[k] + 1e-7f < v[k+1] (boosting_core.cu:400).
    // One thread per unit of 16 consecutive positions: the unit's order
    // entries in two 16-byte loads, all 17 values gathered before any is
    // compared, and the unit's split bits as one 16-bit word (in the free
    // digit-counter array); the words are then stored in the lane-run layout
    // of the resident orders (see ord_slot; a lane run is whole units).
    if (gapOut) {
        uint16_t* gnat16 = reinterpret_cast<uint16_t*>(gnat);
        const int units = (n + 15) >> 4;
        for (int u = tid; u < units; u += kSortThreads) {
            const int k0 = u * 16;
            const uint4 a = *reinterpret_cast<const uint4*>(idx + k0);
            const uint4 b = *reinterpret_cast<const uint4*>(idx + k0 + 8);
            const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            float v[17];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const uint32_t id = (w[i >> 1] >> (16 * (i & 1))) & 0xFFFFu;
                v[i] = k0 + i < n ? __uint_as_float(radix_key_inv(keys[id])) : 0.0f;
            }
            v[16] = k0 + 16 < n ? __uint_as_float(radix_key_inv(keys[idx[k0 + 16]])) : 0.0f;
            uint32_t bits = 0;
#pragma unroll
            for (int i = 0; i < 16; ++i)
                if (k0 + i + 1 < n && __fadd_rn(v[i], 1e-7f) < v[i + 1]) bits |= 1u << i;
            gnat16[u] = static_cast<uint16_t>(bits);
        }
        __syncthreads();
        uint16_t* grow = gapOut + static_cast<size_t>(fl) * gapStride;
        for (int j = tid; j < 2 * L; j += kSortThreads) {
            const int k = (j & 31) * L + 16 * (j >> 5);  // first position of the word
            grow[j] = k < n ? gnat16[k >> 4] : uint16_t(0);
        }
    }
    // Two weight copies: pick each position's copy.  The sweep's gather
    // instruction i of step t reads positions m*L + 16t + i, m = 0..31
    // (lane m); thread g takes that group and assigns its members in turn to
    // the less loaded of their two banks (greedy two-choice, bank loads
    // tracked up to 2 in two bit masks: o1 = banks with load >= 1, o2 = banks
    // with load 2).  The members are read eight at a time, the next eight
    // before the current ones are decided, so no load waits on the chain of
    // decisions.
    if (ordPadded && slotBase > 0) {
        __syncthreads();
        for (int g = tid; g < L; g += kSortThreads) {
            const int kb = 16 * (g >> 4) + (g & 15);
            const int members = kb < n ? min(32, (n - kb + L - 1) / L) : 0;  // kb + m*L < n
            uint32_t o1 = 0, o2 = 0;
            auto read8 = [&](uint32_t (&x)[8], int m0) {
#pragma unroll
                for (int i = 0; i < 8; ++i) x[i] = m0 + i < members ? idx[kb + (m0 + i) * L] : 0u;
            };
            auto decide8 = [&](const uint32_t (&x)[8], int m0) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int m = m0 + i;
                    if (m < members) {
                        const uint32_t off1 = copy1_offset(x[i]);
                        const int b0 = x[i] & 31, b1 = off1 & 31;
                        // copy 1 when its bank is strictly less loaded
                        const uint32_t l0 = ((o1 >> b0) & 1u) + ((o2 >> b0) & 1u);
                        const uint32_t l1 = ((o1 >> b1) & 1u) + ((o2 >> b1) & 1u);
                        const bool one = l1 < l0;
                        const uint32_t bit = 1u << (one ? b1 : b0);
                        o2 |= o1 & bit;
                        o1 |= bit;
                        if (one) idx[kb + m * L] = static_cast<uint16_t>(slotBase + off1);
                    }
                }
            };
            // two register sets of 8 members in turn, each refilled while the
            // other is decided
            uint32_t xa[8], xb[8];
            read8(xa, 0);
            read8(xb, 8);
            decide8(xa, 0);
            read8(xa, 16);
            decide8(xb, 8);
            read8(xb, 24);
            decide8(xa, 16);
            decide8(xb, 24);
        }
        __syncthreads();
    }
    // Sorted sample order (padded rows: lane runs, see ord_slot).  With room
    // in `stage`, the row is first laid out there (each 256-entry block of
    // the row padded by 8 entries, so neither the scattered 16-byte writes
    // nor the reads conflict) and then copied out 512 contiguous bytes per
    // warp instruction; the positions past n carry the zero slot.
    uint16_t* orow = ordOut + static_cast<size_t>(fl) * ordStride;
    if (ordPadded) {
        const int n8 = (n + 7) & ~7;
        if (tid < n8 - n) idx[n + tid] = static_cast<uint16_t>(zero_slot(n, slotBase));
        __syncthreads();
        const int blocks = L / 8;  // 256-entry blocks of the 32 L entries
        if (stage != nullptr && blocks * 264 <= stageCap) {
            const uint32_t zz = static_cast<uint32_t>(zero_slot(n, slotBase)) * 0x10001u;
            for (int k = tid * 8; k < 32 * L; k += kSortThreads * 8) {
                const int o = ord_slot(k, L);
                *reinterpret_cast<uint4*>(stage + o + 8 * (o >> 8)) =
                    k < n8 ? *reinterpret_cast<const uint4*>(idx + k) : make_uint4(zz, zz, zz, zz);
            }
            __syncthreads();
            for (int j = tid; j < blocks * 32; j += kSortThreads) {
                const int b = j >> 5, l = j & 31;
                *reinterpret_cast<uint4*>(orow + b * 256 + l * 8) =
                    *reinterpret_cast<const uint4*>(stage + b * 264 + l * 8);
            }
        } else {
            for (int k = tid * 8; k < n8; k += kSortThreads * 8)
                *reinterpret_cast<uint4*>(orow + ord_slot(k, L)) = *reinterpret_cast<const uint4*>(idx + k);
        }
    } else {
        for (int k = tid; k < n; k += kSortThreads) orow[k] = idx[k];
    }
}

template <int R, bool kFromResp>
__global__ void __launch_bounds__(kSortThreads, 1)
eval_sort_kernel(const vj_haar_feature* __restrict__ feats, int featBegin, int featCount,
                 const uint32_t* __restrict__ sumT, const float* __restrict__ invNorm, int n,
                 const float* __restrict__ resp, uint16_t* __restrict__ ordOut, int64_t ordStride,
                 bool ordPadded, uint16_t* __restrict__ gapOut, int64_t gapStride, int slotBase, int L) {
    constexpr int NP = 1024 * R;
    constexpr bool kPP = sort_ping_pong<R>();
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* keys = reinterpret_cast<uint32_t*>(smem);  // radix keys of the responses, in sample order
    uint16_t* idx = reinterpret_cast<uint16_t*>(keys + NP);   // sorted order after the last pass
    uint16_t* idx2 = idx + NP;                                // second buffer (kPP only)
    uint32_t* cnt = reinterpret_cast<uint32_t*>(idx + (kPP ? 2 * NP : NP));
    __shared__ uint32_t warpTot[32];
    __shared__ vj_haar_feature sfeat;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int fl = blockIdx.x; fl < featCount; fl += gridDim.x) {
        if (kFromResp) {
            const float* row = resp + static_cast<size_t>(fl) * n;
            for (int s = tid; s < n; s += kSortThreads) keys[s] = radix_key(__float_as_uint(row[s]));
        } else {
            if (tid == 0) sfeat = feats[featBegin + fl];
            __syncthreads();
            const vj_haar_feature& f = sfeat;  // read from shared memory (broadcast), not held in registers
            // four samples per iteration keep ~40 independent L2 loads in flight
            for (int s0 = tid; s0 < n; s0 += 4 * kSortThreads) {
                float r[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = s0 + u * kSortThreads;
                    r[u] = s < n ? train_response(f, sumT, n, s, __ldg(invNorm + s)) : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (s0 + u * kSortThreads < n) keys[s0 + u * kSortThreads] = radix_key(__float_as_uint(r[u]));
            }
        }
        for (int p = tid; p < NP; p += kSortThreads) idx[p] = static_cast<uint16_t>(p);
        __syncthreads();

        for (int pass = 0; pass < 4; ++pass) {
            const int shift = pass * 8;
            // with two buffers, even passes read idx and write idx2, odd ones the reverse
            const uint16_t* src = (kPP && (pass & 1)) ? idx2 : idx;
            uint16_t* dst = (kPP && !(pass & 1)) ? idx2 : idx;
            for (int i = tid; i < 256 * kCntStride; i += kSortThreads) cnt[i] = 0;
            __syncthreads();
            // Rank every item among equal digits: items are warp-striped, so
            // (warp, j, lane) order is the current sequence order and ranks are
            // stable.  The leader of each equal-digit group bumps the warp's
            // counter for that digit.
            // Digits first (independent loads), then ranks: peers with the
            // same digit in a step come from 8 ballots, one per digit bit.
            // packed[j]: the item's sample index in the low half (one buffer
            // only) and its rank among equal digits in the high half; with
            // two buffers, items j and j+1 share a word of two 16-bit ranks.
            constexpr int kPacked = kPP ? (R + 1) / 2 : R;
            uint32_t packed[kPacked];
            uint32_t dig[(R + 3) / 4];
#pragma unroll
            for (int j = 0; j < kPacked; ++j) packed[j] = 0;
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int p = warp * 32 * R + j * 32 + lane;
                const uint32_t id = src[p];
                const uint32_t d = id < static_cast<uint32_t>(n) ? (keys[id] >> shift) & 255u : 255u;
                if (!kPP) packed[j] = id;
                if ((j & 3) == 0)
                    dig[j >> 2] = d;
                else
                    dig[j >> 2] |= d << (8 * (j & 3));
            }
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const uint32_t d = __byte_perm(dig[j >> 2], 0u, 0x4440u | static_cast<uint32_t>(j & 3));
                const uint32_t peers = digit_peers(d);
                // every lane reads its digit's counter; once the warp has read,
                // the first lane of each equal-digit group stores the new count
                const uint32_t before = peers & lanemask_lt();
                const uint32_t old = cnt[d * kCntStride + warp];
                __syncwarp();
                if (before == 0) cnt[d * kCntStride + warp] = old + __popc(peers);
                __syncwarp();
                const uint32_t rank = old + __popc(before);
                if (kPP)
                    packed[j >> 1] |= rank << (16 * (j & 1));
                else
                    packed[j] |= rank << 16;
            }
            __syncthreads();
            scan_digit_counters(cnt, warpTot);
            __syncthreads();
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const uint32_t d = __byte_perm(dig[j >> 2], 0u, 0x4440u | static_cast<uint32_t>(j & 3));
                if (kPP) {
                    const uint32_t rank = (packed[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
                    dst[cnt[d * kCntStride + warp] + rank] = src[warp * 32 * R + j * 32 + lane];
                } else {
                    const uint32_t pos = cnt[d * kCntStride + warp] + (packed[j] >> 16);
                    idx[pos] = static_cast<uint16_t>(packed[j] & 0xFFFFu);
                }
            }
            __syncthreads();
        }

        sort_epilogue(keys, idx, cnt, n, fl, ordOut, ordStride, ordPadded, gapOut, gapStride, slotBase, L,
                      reinterpret_cast<uint16_t*>(cnt), 256 * kCntStride * 2);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 1c. The evaluate + stable LSD radix sort with per-thread digit counters, for
//     n <= 1024 * kBlockedMaxR samples.  In every pass thread t takes the R
//     consecutive items [tR, tR + R) of the current sequence (a blocked
//     arrangement), so an item's rank among the thread's items with the same
//     digit is a count the thread keeps itself and no ballot is needed.
//     Digits are 5 bits (32 values); the counters are 16-bit halves of
//     shared-memory words, word row c holding digits c and c + 16 of every
//     thread, and the 32 threads of a warp always touch 32 different banks.
//     An exclusive scan of the counters in (digit, thread) order gives every
//     (digit, thread) pair its first output position; the scatter takes the
//     items again in order and bumps the pair's position per item, so equal
//     digits keep sequence order (stable) and the final order is
//     eval_sort_kernel's.  Seven passes (the last of 2 bits) cover the 32-bit
//     keys.  Positions n..NP-1 carry the largest key, so they stay last.
// ---------------------------------------------------------------------------
constexpr int kDigitBits = 5;
constexpr int kDigitPasses = 7;
constexpr int kCntRows = 16;          // 32 digits, two 16-bit counters a word
constexpr int kCntRow = 1024 + 32;    // a row of 1024 thread words, one pad word per 32
constexpr int kBlockedMaxR = 20;

template <int R>
constexpr size_t blocked_sort_smem_bytes() {
    return static_cast<size_t>(1024 * R) * (4 + 2 + 2) + static_cast<size_t>(kCntRows) * kCntRow * 4 + 16;
}

// Exclusive scan, in place, of the per-thread digit counters in (row, thread)
// order, both halves at once: every total stays below 2^16, so the low halves
// (digits 0..15) never carry into the high ones; the low halves' total is then
// added to every high half, since digits 16..31 follow all of digits 0..15.
// Thread t takes the 16 consecutive words [16t, 16t + 16) of that order; with
// one pad word per 32, the 32 lanes of a warp read 32 different banks.
__device__ __forceinline__ void scan_thread_counters(uint32_t* cnt, uint32_t* warpTot, uint32_t* blockTotal) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int t0 = (tid & 63) * 16;
    uint32_t* base = cnt + (tid >> 6) * kCntRow + t0 + (t0 >> 5);
    uint32_t v[16];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        v[k] = base[k];
        sum += v[k];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = warpTot[lane];
        uint32_t x = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        warpTot[lane] = x - t;
        if (lane == 31) *blockTotal = x;
    }
    __syncthreads();
    uint32_t run = warpTot[warp] + incl - sum + ((*blockTotal & 0xFFFFu) << 16);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        base[k] = run;
        run += v[k];
    }
}

// Four consecutive items' sample indices (16 bits each) of a blocked pass:
// in pass 0 the positions themselves (the sample order), later from the
// source buffer.
__device__ __forceinline__ uint2 load_four(const uint2* src4, int pass, int pos, int j) {
    if (pass == 0) {
        const uint32_t lo = static_cast<uint32_t>(pos) * 0x10001u + 0x10000u;
        return make_uint2(lo, lo + 0x20002u);
    }
    return src4[j / 4];
}

template <int R, bool kFromResp>
__global__ void __launch_bounds__(kSortThreads, 1)
eval_sort_blocked_kernel(const vj_haar_feature* __restrict__ feats, int featBegin, int featCount,
                         const uint32_t* __restrict__ sumT, const float* __restrict__ invNorm, int n,
                         const float* __restrict__ resp, uint16_t* __restrict__ ordOut, int64_t ordStride,
                         bool ordPadded, uint16_t* __restrict__ gapOut, int64_t gapStride, int slotBase, int L) {
    static_assert(R % 4 == 0 && R <= kBlockedMaxR, "a multiple of 4 items per thread, at most kBlockedMaxR");
    constexpr int NP = 1024 * R;
    constexpr int kPk = (R + 5) / 6;  // words of six 5-bit digits
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* keys = reinterpret_cast<uint32_t*>(smem);     // radix keys in sample order
    uint16_t* idxA = reinterpret_cast<uint16_t*>(keys + NP);
    uint16_t* idxB = idxA + NP;                              // the sorted order after the last pass
    uint32_t* cnt = reinterpret_cast<uint32_t*>(idxB + NP);  // [kCntRows][kCntRow]
    uint32_t* blockTotal = cnt + kCntRows * kCntRow;
    __shared__ uint32_t warpTot[32];
    __shared__ vj_haar_feature sfeat;
    const int tid = threadIdx.x;
    uint32_t* ccol = cnt + tid + (tid >> 5);  // this thread's counter word of row 0

    for (int fl = blockIdx.x; fl < featCount; fl += gridDim.x) {
        if (kFromResp) {
            const float* row = resp + static_cast<size_t>(fl) * n;
            for (int s = tid; s < NP; s += kSortThreads) keys[s] = s < n ? radix_key(__float_as_uint(row[s])) : ~0u;
        } else {
            if (tid == 0) sfeat = feats[featBegin + fl];
            __syncthreads();
            const vj_haar_feature& f = sfeat;
            // four samples per thread in flight; each corner a feature's
            // rectangles share is loaded once (corner_sharing); with n even
            // and aligned tables, a thread's samples come in consecutive
            // pairs and each corner is one 8-byte load for a pair
            const bool vec2 = (n & 1) == 0 && (reinterpret_cast<uintptr_t>(sumT) & 7) == 0 &&
                              (reinterpret_cast<uintptr_t>(invNorm) & 7) == 0;
            auto eval = [&](auto shape) {
                constexpr int S = decltype(shape)::value;
                if constexpr (S != 0) {
                if (vec2) {
                    for (int s0 = 2 * tid; s0 < NP; s0 += 4 * kSortThreads) {
                        float2 r[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int s = s0 + u * 2 * kSortThreads;
                            r[u] = s < n ? train_response2<S>(f, sumT, n, s,
                                                              __ldg(reinterpret_cast<const float2*>(invNorm + s)))
                                         : make_float2(0.0f, 0.0f);
                        }
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int s = s0 + u * 2 * kSortThreads;
                            if (s < NP)
                                *reinterpret_cast<uint2*>(keys + s) =
                                    s < n ? make_uint2(radix_key(__float_as_uint(r[u].x)), radix_key(__float_as_uint(r[u].y)))
                                          : make_uint2(~0u, ~0u);
                        }
                    }
                    return;
                }
                }
                for (int s0 = tid; s0 < NP; s0 += 4 * kSortThreads) {
                    float r[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = s0 + u * kSortThreads;
                        r[u] = s < n ? train_response_shared<S>(f, sumT, n, s, __ldg(invNorm + s)) : 0.0f;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = s0 + u * kSortThreads;
                        if (s < NP) keys[s] = s < n ? radix_key(__float_as_uint(r[u])) : ~0u;
                    }
                }
            };
            switch (corner_sharing(f)) {
                case 1: eval(std::integral_constant<int, 1>()); break;
                case 2: eval(std::integral_constant<int, 2>()); break;
                case 3: eval(std::integral_constant<int, 3>()); break;
                default: eval(std::integral_constant<int, 0>()); break;
            }
        }
        __syncthreads();

        for (int pass = 0; pass < kDigitPasses; ++pass) {
            const int shift = pass * kDigitBits;
            // pass 0 takes the sample order; even passes write B, odd ones A
            // a thread's R indices as R/4 8-byte words: 40 bytes apart, so a
            // half-warp's 16 loads cover the 32 banks once
            const uint2* src4 = reinterpret_cast<const uint2*>((pass & 1) ? idxB : idxA) + tid * (R / 4);
            uint16_t* dst = (pass & 1) ? idxA : idxB;
#pragma unroll
            for (int c = 0; c < kCntRows; ++c) ccol[c * kCntRow] = 0;
            uint32_t dg[kPk];
#pragma unroll
            for (int c = 0; c < kPk; ++c) dg[c] = 0;
#pragma unroll
            for (int j = 0; j < R; j += 4) {
                // pass 0 takes the sample order: a thread's four keys are
                // consecutive, one 16-byte load (80 bytes apart across the
                // warp, so each quarter-warp covers the 32 banks once)
                uint32_t k[4];
                if (pass == 0) {
                    const uint4 k4 = *reinterpret_cast<const uint4*>(keys + tid * R + j);
                    k[0] = k4.x, k[1] = k4.y, k[2] = k4.z, k[3] = k4.w;
                } else {
                    const uint2 four = src4[j / 4];
#pragma unroll
                    for (int h = 0; h < 4; ++h) k[h] = keys[((h < 2 ? four.x : four.y) >> (16 * (h & 1))) & 0xFFFFu];
                }
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const uint32_t d = (k[h] >> shift) & 31u;
                    ccol[(d & 15u) * kCntRow] += 1u << (d & 16u);
                    dg[(j + h) / 6] |= d << (5 * ((j + h) % 6));
                }
            }
            __syncthreads();
            scan_thread_counters(cnt, warpTot, blockTotal);
            __syncthreads();
#pragma unroll
            for (int j = 0; j < R; j += 4) {
                const uint2 four = load_four(src4, pass, tid * R + j, j);
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const uint32_t id = ((h < 2 ? four.x : four.y) >> (16 * (h & 1))) & 0xFFFFu;
                    const uint32_t d = (dg[(j + h) / 6] >> (5 * ((j + h) % 6))) & 31u;
                    uint32_t* cw = ccol + (d & 15u) * kCntRow;
                    const uint32_t w = *cw;
                    *cw = w + (1u << (d & 16u));
                    dst[(w >> (d & 16u)) & 0xFFFFu] = static_cast<uint16_t>(id);
                }
            }
            __syncthreads();
        }
        sort_epilogue(keys, idxB, cnt, n, fl, ordOut, ordStride, ordPadded, gapOut, gapStride, slotBase, L,
                      reinterpret_cast<uint16_t*>(cnt), kCntRows * kCntRow * 2);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 1b. The same evaluate + stable LSD radix sort for 32,768 < n <= 65,535
//     samples, which do not fit on chip.  Each CTA keeps its feature's keys
//     and sample indices in a private global scratch (12 bytes per position:
//     two key and two index buffers; about 0.8 MB per CTA at 65,536
//     positions, so the scratch of all CTAs stays mostly in L2) and moves the
//     keys with the indices, so every read of a pass is coalesced; the ranks
//     among equal digits (2 bytes per position) stay in shared memory.  Items
//     are warp-contiguous as in eval_sort_kernel (position
//     warp * 32R + 32j + lane), ranks come from the same ballots, and the
//     outputs (order, split bitmask, layouts) are the same.  Positions from n
//     up to 1024R carry the largest key and sort last.
// ---------------------------------------------------------------------------
constexpr int kOnChipSortMax = 32768;
constexpr int kLargeSortMaxR = 64;  // 65,536 positions per feature
__host__ __device__ __forceinline__ int large_sort_r(int n) { return (n + 1023) / 1024; }
inline size_t large_sort_smem_bytes(int R) {
    return static_cast<size_t>(256 * kCntStride) * 4 + static_cast<size_t>(1024 * R) * 2;
}

template <bool kFromResp>
__global__ void __launch_bounds__(kSortThreads, 1)
eval_sort_large_kernel(const vj_haar_feature* __restrict__ feats, int featBegin, int featCount,
                       const uint32_t* __restrict__ sumT, const float* __restrict__ invNorm, int n,
                       const float* __restrict__ resp, uint16_t* __restrict__ ordOut, int64_t ordStride,
                       bool ordPadded, uint16_t* __restrict__ gapOut, int64_t gapStride, int L, int R,
                       uint32_t* __restrict__ keyScratch, uint16_t* __restrict__ idxScratch) {
    const int NP = 1024 * R;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem);           // digit counters; later the split-bit words
    uint16_t* rankS = reinterpret_cast<uint16_t*>(cnt + 256 * kCntStride);  // rank among equal digits
    __shared__ uint32_t warpTot[32];
    __shared__ vj_haar_feature sfeat;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gapWords = (n + 31) >> 5;
    uint32_t* keyA = keyScratch + static_cast<size_t>(blockIdx.x) * 2 * NP;
    uint32_t* keyB = keyA + NP;
    uint16_t* idxA = idxScratch + static_cast<size_t>(blockIdx.x) * 2 * NP;
    uint16_t* idxB = idxA + NP;

    for (int fl = blockIdx.x; fl < featCount; fl += gridDim.x) {
        // radix keys in sample order
        if (kFromResp) {
            const float* row = resp + static_cast<size_t>(fl) * n;
            for (int s = tid; s < NP; s += kSortThreads) keyA[s] = s < n ? radix_key(__float_as_uint(row[s])) : ~0u;
        } else {
            if (tid == 0) sfeat = feats[featBegin + fl];
            __syncthreads();
            const vj_haar_feature& f = sfeat;
            for (int s0 = tid; s0 < NP; s0 += 4 * kSortThreads) {
                float r[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = s0 + u * kSortThreads;
                    r[u] = s < n ? train_response(f, sumT, n, s, __ldg(invNorm + s)) : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = s0 + u * kSortThreads;
                    if (s < NP) keyA[s] = s < n ? radix_key(__float_as_uint(r[u])) : ~0u;
                }
            }
        }
        __syncthreads();

        for (int pass = 0; pass < 4; ++pass) {
            const int shift = pass * 8;
            const uint32_t* ks = (pass & 1) ? keyB : keyA;
            uint32_t* kd = (pass & 1) ? keyA : keyB;
            const uint16_t* is = (pass & 1) ? idxB : idxA;
            uint16_t* id = (pass & 1) ? idxA : idxB;
            for (int i = tid; i < 256 * kCntStride; i += kSortThreads) cnt[i] = 0;
            __syncthreads();
            // ranks among equal digits, in sequence order (warp-contiguous items)
#pragma unroll 4
            for (int j = 0; j < R; ++j) {
                const int p = warp * 32 * R + j * 32 + lane;
                const uint32_t d = (ks[p] >> shift) & 255u;
                const uint32_t peers = digit_peers(d);
                const uint32_t before = peers & lanemask_lt();
                const uint32_t old = cnt[d * kCntStride + warp];
                __syncwarp();
                if (before == 0) cnt[d * kCntStride + warp] = old + __popc(peers);
                __syncwarp();
                rankS[p] = static_cast<uint16_t>(old + __popc(before));
            }
            __syncthreads();
            scan_digit_counters(cnt, warpTot);
            __syncthreads();
#pragma unroll 4
            for (int j = 0; j < R; ++j) {
                const int p = warp * 32 * R + j * 32 + lane;
                const uint32_t key = ks[p];
                const uint32_t d = (key >> shift) & 255u;
                const uint32_t pos = cnt[d * kCntStride + warp] + rankS[p];
                kd[pos] = key;
                id[pos] = pass == 0 ? static_cast<uint16_t>(p) : is[p];
            }
            __syncthreads();
        }
        // after four passes the sorted keys and indices are in keyA / idxA

        if (gapOut) {
            uint32_t* gnat = cnt;
            for (int k0 = warp * 32; k0 < gapWords * 32; k0 += kSortThreads) {
                const int k = k0 + lane;
                const float v0 = k < n ? __uint_as_float(radix_key_inv(keyA[k])) : 0.0f;
                float v1 = __shfl_down_sync(0xffffffffu, v0, 1);
                if (lane == 31 && k + 1 < n) v1 = __uint_as_float(radix_key_inv(keyA[k + 1]));
                const uint32_t bits = __ballot_sync(0xffffffffu, k + 1 < n && __fadd_rn(v0, 1e-7f) < v1);
                if (lane == 0) gnat[k0 >> 5] = bits;
            }
            __syncthreads();
            uint16_t* grow = gapOut + static_cast<size_t>(fl) * gapStride;
            for (int j = tid; j < 2 * L; j += kSortThreads) {
                const int k = (j & 31) * L + 16 * (j >> 5);
                grow[j] = k < n ? static_cast<uint16_t>(gnat[k >> 5] >> (k & 31)) : uint16_t(0);
            }
        }
        uint16_t* orow = ordOut + static_cast<size_t>(fl) * ordStride;
        if (ordPadded) {
            // lane-run layout; positions from n to the next multiple of 8 hold
            // the zero slot (one weight copy: slot n)
            const int n8 = (n + 7) & ~7;
            const uint32_t zs = static_cast<uint32_t>(zero_slot(n, 0));
            for (int k = tid * 8; k < n8; k += kSortThreads * 8) {
                uint4 v = *reinterpret_cast<const uint4*>(idxA + k);
                if (k + 8 > n) {
                    uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (k + e >= n) w4[e >> 1] = (w4[e >> 1] & ~(0xFFFFu << (16 * (e & 1)))) | (zs << (16 * (e & 1)));
                    v = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
                *reinterpret_cast<uint4*>(orow + ord_slot(k, L)) = v;
            }
        } else {
            for (int k = tid; k < n; k += kSortThreads) orow[k] = idxA[k];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Per-round weight preparation: signed weights (+w positive, -w negative,
// +-0 inactive), totals and the candidate window.
// ---------------------------------------------------------------------------
// With wShadow / aShadow given (the resident search), the kernel also decides
// whether last round's per-feature bounds may prune this round's sweep: only
// when the weights are bit for bit what the last vj_round_update left
// (wShadow) and the active mask is what the last search saw (aShadow), i.e.
// nothing but that update changed them.
//
// One thread per sample over ceil(n / 1024) blocks; each block writes its
// totals (a fixed shuffle tree) to part[block], and the last block to finish
// adds the partials in block order, so the totals do not depend on timing.
struct PrepPartial {
    double tp, tn;
    int np, nn, diff, pad;
};
constexpr int kPrepMaxBlocks = 64;  // 65,536 samples

__global__ void __launch_bounds__(1024)
prep_round_kernel(const int8_t* __restrict__ label, const uint8_t* __restrict__ active,
                  const float* __restrict__ weight, int n, float* __restrict__ wsg,
                  RoundParams* __restrict__ prm, const float* __restrict__ wShadow, uint8_t* __restrict__ aShadow,
                  const PruneState* __restrict__ ps, const int* gate, PrepPartial* __restrict__ part,
                  unsigned int* __restrict__ done) {
    if (gate_closed(gate)) return;
    __shared__ double sp[32], sn[32];
    __shared__ int cp[32], cn[32], cd[32];
    __shared__ bool lastBlock;
    double tp = 0.0, tn = 0.0;
    int np = 0, nn = 0, diff = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) wsg[n] = 0.0f;  // the zero slot of one-copy orders
    if (i < n) {
        const bool act = active == nullptr || active[i] != 0;
        const float wi = weight[i];
        if (wShadow) {
            diff = __float_as_uint(wi) != __float_as_uint(wShadow[i]);
            const uint8_t a = act ? 1 : 0;
            diff |= aShadow[i] != a;
            aShadow[i] = a;
        }
        const float w = act ? wi : 0.0f;
        const bool pos = label[i] > 0;
        wsg[i] = pos ? w : -w;
        if (act) {
            if (pos) {
                tp = static_cast<double>(w);
                np = 1;
            } else {
                tn = static_cast<double>(w);
                nn = 1;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        tp += __shfl_down_sync(0xffffffffu, tp, o);
        tn += __shfl_down_sync(0xffffffffu, tn, o);
        np += __shfl_down_sync(0xffffffffu, np, o);
        nn += __shfl_down_sync(0xffffffffu, nn, o);
        diff |= __shfl_down_sync(0xffffffffu, diff, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sp[warp] = tp;
        sn[warp] = tn;
        cp[warp] = np;
        cn[warp] = nn;
        cd[warp] = diff;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        PrepPartial b{0.0, 0.0, 0, 0, 0, 0};
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) {
            b.tp += sp[k];
            b.tn += sn[k];
            b.np += cp[k];
            b.nn += cn[k];
            b.diff |= cd[k];
        }
        part[blockIdx.x] = b;
        __threadfence();
        lastBlock = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (lastBlock && threadIdx.x == 0) {
        __threadfence();
        double TP = 0.0, TN = 0.0;
        int NP = 0, NN = 0, changed = 0;
        for (int k = 0; k < static_cast<int>(gridDim.x); ++k) {
            TP += __ldcg(&part[k].tp);
            TN += __ldcg(&part[k].tn);
            NP += __ldcg(&part[k].np);
            NN += __ldcg(&part[k].nn);
            changed |= __ldcg(&part[k].diff);
        }
        *done = 0u;  // ready for the next launch
        const double u = 5.9604644775390625e-08;
        auto gamma = [&](int k) { return static_cast<double>(k) * u / (1.0 - static_cast<double>(k) * u); };
        const double W = TP + TN;
        // |sequential FP32 error - exact| for either parity (see the header).
        const double bcpu = 2.0 * gamma(NP + 2) * TP + 2.0 * gamma(NN + 2) * TN + 4.0 * u * W;
        // fast pass: a position's prefix is fl(E + fl(b + s)) with s a sum of
        // <= 16 terms (15 roundings), b the lane's Kahan carry of its earlier
        // 16-term step sums (15 + 2 roundings over the lane's mass), E the
        // warp-scanned sum of the earlier lanes' carries (17 + 5 over theirs),
        // then 1 + 1 additions and the final difference: <= 25 u W, taken as 64.
        const double bfast = 64.0 * u * W;
        const double window = 2.0 * (bcpu + bfast) * 1.01 + 1e-30;
        prm->tp = static_cast<float>(TP);
        prm->tn = static_cast<float>(TN);
        prm->w = static_cast<float>(W);
        prm->window = static_cast<float>(window);
        prm->fastMinBits = 0x7F800000u;
        prm->ncand = 0;
        prm->winner = ~0ull;
        prm->np = NP;
        prm->nn = NN;
        prm->status = 0;
        prm->bfast = __double2float_ru(bfast);
        prm->pruneOK = (wShadow && ps->valid && !changed) ? 1 : 0;
        prm->lbScale = prm->pruneOK ? ps->scale : 0.0f;
        prm->nextFeat = 0;
        prm->swept = 0;
    }
}

// ---------------------------------------------------------------------------
// 2. Fast sweep: one warp per feature, minimum weighted error to within the
//    bound used for the window.
// ---------------------------------------------------------------------------
constexpr int kSweepChunk = 2;  // features a warp takes from the shared counter at once

template <bool kSmemW, int TPB>
__global__ void __launch_bounds__(TPB, 1024 / TPB)
sweep_kernel(const uint16_t* __restrict__ ord, int64_t ordStride, const uint16_t* __restrict__ gap,
             int64_t gapStride, const float* __restrict__ wsgG, int n, int slotBase, int L, int featCount,
             const uint8_t* __restrict__ usedMask, RoundParams* __restrict__ prm,
             float* __restrict__ fastErr, float* __restrict__ lb, unsigned long long* __restrict__ sweptTotal,
             const int* gate) {
    if (gate_closed(gate)) return;
    extern __shared__ float wsgS[];
    const float* wsg = wsgG;
    if (kSmemW) {
        fill_weights(wsgS, wsgG, n, slotBase);
        __syncthreads();
        wsg = wsgS;
    }
    // With P(k) the prefix sum of signed weights over the sorted order, the
    // two parities' errors at split k are T+ - P(k) and T- + P(k), so a
    // feature's best error is min(T+ - max P, T- + min P) over valid splits.
    //
    // One warp per feature at a time.  Lane l walks its run of L sorted
    // positions [l*L, (l+1)*L) 16 at a time (two 16-byte slot loads, 16 split
    // bits) with a lane-local running sum, Kahan-compensated across steps, and
    // keeps the minimum and maximum of that sum over its valid splits; at the
    // feature's end one warp scan gives each lane the sum of the runs before
    // its own, which is added once.  Rounding is monotone, so
    // min_i fl(b + s_i) = fl(b + min_i s_i).  Padding positions carry the zero
    // slot and no split bit, so no position needs a mask.  A warp walks the
    // (feature, step) items of the features it takes; the loads of the next
    // item are issued before the current one is processed, across feature
    // boundaries.
    //
    // Features come in chunks of kSweepChunk from a counter shared by all
    // warps.  When a warp reaches a feature it compares the feature's bound -
    // a lower bound of its exact best error under this round's weights: last
    // round's fast error minus the fast pass's error bound, or last round's
    // bound, times the update's factor lbScale - with the round's running
    // minimum of the fast errors.  A feature whose bound exceeds that minimum
    // plus the candidate window has exact error above (minimum exact error)
    // + 2 x (the reference's FP32 error bound), so it cannot be the
    // reference's pick and is not streamed: its fast error is +inf (no
    // candidate) and its bound is kept for the next round.  Streamed features
    // leave fresh bounds.
    const float TP = prm->tp, TN = prm->tn;
    const float window = prm->window, bfast = prm->bfast, scale = prm->lbScale;
    const bool prune = prm->pruneOK != 0;
    const int lane = threadIdx.x & 31;
    const int spf = L >> 4;  // steps per feature
    const uint32_t z = static_cast<uint32_t>(zero_slot(n, slotBase)) * 0x10001u;
    const volatile unsigned int* runMinBits = &prm->fastMinBits;
    float runMin = INFINITY;  // the warp's view of the running minimum (warp-uniform)
    int qBase = 0;
    unsigned qMask = 0;  // features of the warp's chunk not yet reached
    int swept = 0;
    // The next feature to stream (warp-uniform), or -1 when none is left.
    auto next_feature = [&]() -> int {
        for (;;) {
            if (qMask == 0) {
                int c0 = 0;
                if (lane == 0) c0 = static_cast<int>(atomicAdd(&prm->nextFeat, static_cast<unsigned>(kSweepChunk)));
                c0 = __shfl_sync(0xffffffffu, c0, 0);
                if (c0 >= featCount) return -1;
                qBase = c0;
                const int k = min(kSweepChunk, featCount - c0);
                qMask = (1u << k) - 1u;
            }
            runMin = fminf(runMin, __uint_as_float(*runMinBits));
            const float lim = __fadd_ru(runMin, window);
            const bool mine = lane < kSweepChunk && ((qMask >> lane) & 1u);
            bool keep = false, used = false;
            float bound = 0.0f;
            if (mine) {
                const int c = qBase + lane;
                used = usedMask != nullptr && usedMask[c] != 0;
                if (prune) bound = __fmul_rd(lb[c], scale);
                keep = !used && !(bound > lim);
            }
            const unsigned km = __ballot_sync(0xffffffffu, keep);
            const int first = km ? __ffs(km) - 1 : 32;
            // the chunk's features before the first one kept are not streamed;
            // their bounds (also those of used features, which a caller may
            // clear later) carry over to the next round
            if (mine && lane < first) {
                const int c = qBase + lane;
                fastErr[c] = INFINITY;
                lb[c] = bound;
            }
            if (km) {
                qMask &= ~((2u << first) - 1u);
                return qBase + first;
            }
            qMask = 0;
        }
    };
    // Used features are skipped when reached, so no load waits on the mask.
    // A cursor is a (feature, step) item with the addresses of its order and
    // bitmask words; stepping within a feature only moves the addresses.
    struct Cursor {
        int f, t, k0;
        const uint16_t* row;  // ord_slot(k0, L) of this lane
        const uint16_t* gw;   // gap_word(k0, L) of this lane
    };
    auto start = [&](Cursor& c, int f) {
        c.f = f;
        c.t = 0;
        c.k0 = lane * L;
        if (f >= 0) {
            c.row = ord + static_cast<size_t>(f) * ordStride + lane * 8;
            c.gw = gap + static_cast<size_t>(f) * gapStride + lane;
        }
    };
    auto load = [&](const Cursor& c, uint4& a, uint4& b, uint32_t& g) {
        a = b = make_uint4(z, z, z, z);
        g = 0;
        if (c.f < 0) return;
        if (c.k0 < n) a = __ldg(reinterpret_cast<const uint4*>(c.row));
        if (c.k0 + 8 < n) b = __ldg(reinterpret_cast<const uint4*>(c.row + 256));
        if (c.k0 < n - 1) g = __ldg(c.gw);
    };
    auto advance = [&](Cursor& c) {
        if (c.f < 0) return;
        if (++c.t == spf) {
            start(c, next_feature());
        } else {
            c.k0 += 16;
            c.row += 512;
            c.gw += 32;
        }
    };
    // The loop is unrolled twice so that the two sets of item registers
    // alternate between "being processed" and "being loaded" without copies.
    Cursor ld;  // the item being loaded
    start(ld, next_feature());
    int pf = ld.f;                   // feature of the item being processed, -1 at the end
    bool plast = ld.t == spf - 1;    // the item is its feature's last step
    uint4 a0, b0, a1, b1;
    uint32_t g0, g1;
    load(ld, a0, b0, g0);
    advance(ld);
    float carry = 0.0f, comp = 0.0f, pmin = INFINITY, pmax = -INFINITY;
    auto step = [&](const uint4& ca, const uint4& cb, const uint32_t cg, uint4& na, uint4& nb, uint32_t& ng) {
        const int qf = ld.f;
        const bool qlast = ld.t == spf - 1;
        load(ld, na, nb, ng);
        advance(ld);
        const uint32_t w8[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
        float s = 0.0f, lmin = INFINITY, lmax = -INFINITY;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            s = __fadd_rn(s, wsg[(w8[i >> 1] >> (16 * (i & 1))) & 0xFFFFu]);
            if ((cg >> i) & 1u) {
                lmin = fminf(lmin, s);
                lmax = fmaxf(lmax, s);
            }
        }
        // a step without a valid split leaves lmin = +inf and lmax = -inf,
        // which the carry keeps infinite and the merge ignores
        pmin = fminf(pmin, __fadd_rn(carry, lmin));
        pmax = fmaxf(pmax, __fadd_rn(carry, lmax));
        {
            const float y = __fsub_rn(s, comp);
            const float u = __fadd_rn(carry, y);
            comp = __fsub_rn(__fsub_rn(u, carry), y);
            carry = u;
        }
        if (plast) {
            // exclusive prefix of the lanes' run sums
            float incl = carry;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl = __fadd_rn(incl, y);
            }
            float excl = __shfl_up_sync(0xffffffffu, incl, 1);
            if (lane == 0) excl = 0.0f;
            float lo = INFINITY, hi = -INFINITY;
            if (pmax > -INFINITY) {
                lo = __fadd_rn(excl, pmin);
                hi = __fadd_rn(excl, pmax);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            float best = INFINITY;
            if (hi > -INFINITY) best = fmaxf(fminf(__fsub_rn(TP, hi), __fadd_rn(TN, lo)), 0.0f);
            if (lane == 0) {
                fastErr[pf] = best;
                // exact best error >= fast error - bfast; +inf for no valid split,
                // which no later round of the stage can change
                lb[pf] = fmaxf(__fsub_rd(best, bfast), 0.0f);
                if (best < runMin) atomicMin(&prm->fastMinBits, __float_as_uint(best));
                ++swept;
            }
            runMin = fminf(runMin, best);
            carry = comp = 0.0f;
            pmin = INFINITY;
            pmax = -INFINITY;
        }
        pf = qf;
        plast = qlast;
    };
    while (pf >= 0) {
        step(a0, b0, g0, a1, b1, g1);
        if (pf < 0) break;
        step(a1, b1, g1, a0, b0, g0);
    }
    if (lane == 0 && swept) {
        atomicAdd(&prm->swept, swept);
        atomicAdd(sweptTotal, static_cast<unsigned long long>(swept));
    }
}

// ---------------------------------------------------------------------------
// 3. Candidate selection.
// ---------------------------------------------------------------------------
__global__ void select_candidates_kernel(const float* __restrict__ fastErr, int featCount,
                                         RoundParams* __restrict__ prm, int* __restrict__ cand, const int* gate) {
    if (gate_closed(gate)) return;
    const float lim = __fadd_rn(__uint_as_float(prm->fastMinBits), prm->window);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < featCount; f += gridDim.x * blockDim.x) {
        const float e = fastErr[f];
        if (e <= lim && e < INFINITY) cand[atomicAdd(&prm->ncand, 1)] = f;
    }
}

// ---------------------------------------------------------------------------
// 4. Exact replay of runCpuWeakSearch (main.cu:626-678) for each candidate:
//    sequential FP32 totals over the sorted order, then the sequential sweep
//    with the CPU's update rule (lower err wins; at equal err parity +1
//    replaces parity -1).
// ---------------------------------------------------------------------------
constexpr int kRefinePairs = kRefineWarps / 2;  // candidates a block takes at once

// Named barrier of the two warps of pair `pair` (barrier 0 is __syncthreads).
__device__ __forceinline__ void pair_sync(int pair) {
    asm volatile("bar.sync %0, 64;" ::"r"(pair + 1) : "memory");
}

template <bool kSmemW>
__global__ void __launch_bounds__(kRefineThreads)
refine_kernel(const uint16_t* __restrict__ ord, int64_t ordStride, const uint16_t* __restrict__ gap,
              int64_t gapStride, const float* __restrict__ wsgG, int n, int slotBase, int L,
              RoundParams* __restrict__ prm,
              const int* __restrict__ cand, int8_t* __restrict__ refParity, int* __restrict__ refSplit,
              unsigned long long* __restrict__ candKey, float2* __restrict__ prefix, int64_t prefixStride,
              const int* gate) {
    if (gate_closed(gate)) return;
    if (static_cast<int>(blockIdx.x) * kRefinePairs >= prm->ncand) return;  // no candidate in this block
    extern __shared__ float wsgS[];
    // per pair, two chunk buffers of 256 positions: first the (positive,
    // negative) addends of each position's sample, then, in place, the left
    // sums after it
    __shared__ __align__(16) float2 pre[kRefinePairs][2][256];
    __shared__ float2 totals[kRefinePairs];
    __shared__ unsigned long long pairBest[kRefinePairs];
    const float* wsg = wsgG;
    if (kSmemW) {
        fill_weights(wsgS, wsgG, n, slotBase);
        __syncthreads();
        wsg = wsgS;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int pr = w >> 1;          // the pair of warps this warp belongs to
    const bool chainer = (w & 1);   // second warp of the pair: runs the chains
    const int gw = blockIdx.x * kRefineWarps + 2 * pr;  // row of `prefix` the pair uses
    const int nc = prm->ncand;
    const int chunks = (n + 255) / 256;
    // Two warps per candidate feature.  The first streams the feature's
    // sorted order 256 positions at a time (one coalesced 16-byte load per
    // lane, issued a chunk ahead), gathers the signed weights and stores each
    // position's two addends (|w| to its class's sum, +0.0f to the other) in
    // order into one of the pair's two chunk buffers, while lane 0 of the
    // second warp replays the reference's sequential FP32 additions
    // (main.cu:626-678) over the previous chunk in the other buffer and the
    // second warp copies that chunk's left sums to the pair's row of
    // `prefix`.  Inactive samples carry a zero weight and the accumulator of
    // the other class adds +0.0f: both leave an FP32 sum of non-negative
    // terms unchanged, exactly as skipping them does.
    for (int c = blockIdx.x * kRefinePairs + pr; c < nc; c += gridDim.x * kRefinePairs) {
        const int f = cand[c];
        const uint16_t* row = ord + static_cast<size_t>(f) * ordStride;
        const uint16_t* grow = gap + static_cast<size_t>(f) * gapStride;
        float2* prow = prefix + static_cast<size_t>(gw) * prefixStride;
        auto load = [&](int base) {
            const int k0 = base + lane * 8;
            return (k0 < n) ? __ldg(reinterpret_cast<const uint4*>(row + ord_slot(k0, L))) : make_uint4(0, 0, 0, 0);
        };
        auto gather = [&](int base, const uint4& v, float2* buf) {
            const int k0 = base + lane * 8;
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
            float4* st = reinterpret_cast<float4*>(buf + lane * 8);
#pragma unroll
            for (int h = 0; h < 8; h += 2) {
                float ap[2], an[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const bool in = k0 + h + u < n;
                    const uint32_t id = in ? ((w4[(h + u) >> 1] >> (16 * ((h + u) & 1))) & 0xFFFFu) : 0u;
                    const float e = in ? wsg[id] : 0.0f;
                    const bool neg = signbit(e);
                    ap[u] = neg ? 0.0f : fabsf(e);
                    an[u] = neg ? fabsf(e) : 0.0f;
                }
                st[h >> 1] = make_float4(ap[0], an[0], ap[1], an[1]);
            }
        };
        // One sequential pass: the left sums after every position, in sorted
        // order.  Carried on to the last position, the same chain gives the
        // totals: the reference adds the same weights in the same order for
        // both (main.cu:626-645).  Step i: the gatherer fills chunk i's buffer
        // while the chainer sums chunk i - 1.
        float tp = 0.0f, tn = 0.0f;
        uint4 v = chainer ? make_uint4(0, 0, 0, 0) : load(0);
        for (int i = 0; i <= chunks; ++i) {
            if (!chainer) {
                if (i < chunks) {
                    const uint4 vn = load((i + 1) * 256);
                    gather(i * 256, v, pre[pr][i & 1]);
                    v = vn;
                }
            } else if (i > 0) {
                const int base = (i - 1) * 256;
                float2* buf = pre[pr][(i - 1) & 1];
                if (lane == 0) {
                    float4* st = reinterpret_cast<float4*>(buf);
                    for (int j0 = 0; j0 < 128; j0 += 8) {
                        float4 q[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) q[j] = st[j0 + j];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const float p0 = __fadd_rn(tp, q[j].x), n0 = __fadd_rn(tn, q[j].y);
                            tp = __fadd_rn(p0, q[j].z);
                            tn = __fadd_rn(n0, q[j].w);
                            q[j] = make_float4(p0, n0, tp, tn);
                        }
#pragma unroll
                        for (int j = 0; j < 8; ++j) st[j0 + j] = q[j];
                    }
                }
                __syncwarp();
                // the chunk's left sums to the pair's row, coalesced
                const int lim = min(256, n - 1 - base);  // positions scored: 0 .. n-2
                for (int q = lane; q < lim; q += 32) prow[base + q] = buf[q];
            }
            pair_sync(pr);
        }
        if (chainer && lane == 0) totals[pr] = make_float2(tp, tn);
        pair_sync(pr);
        tp = totals[pr].x;
        tn = totals[pr].y;
        // Scoring, both warps, chunks alternating between them, every lane
        // over its positions.  The reference's update rule over the
        // candidates in split order (lower error replaces; at equal error
        // parity +1 replaces parity -1) picks the lexicographic minimum of
        // (error, parity +1 before -1, split index); errors are >= +0, so the
        // float bits order like the values and the triple packs into one key.
        unsigned long long best = ~0ull;
        // the 8 split bits of positions k0..k0+7 (one lane run, one bitmask
        // word) and the left sums at the valid ones; issued a chunk ahead
        auto sload = [&](int base, float2 (&lv)[8]) -> uint32_t {
            const int k0 = base + lane * 8;
            uint32_t g = 0;
            if (k0 < n - 1) {
                const int l = k0 / L, r = k0 - l * L;
                g = (static_cast<uint32_t>(__ldg(grow + (r >> 4) * 32 + l)) >> (r & 15)) & 0xFFu;  // gap_word
            }
#pragma unroll
            for (int h = 0; h < 8; ++h) lv[h] = ((g >> h) & 1u) ? prow[k0 + h] : make_float2(0.0f, 0.0f);
            return g;
        };
        const int first = chainer ? 256 : 0;
        float2 lc[8];
        uint32_t gc = sload(first, lc);
        for (int base = first; base < n - 1; base += 512) {
            float2 ln[8];
            const uint32_t gn = sload(base + 512, ln);
            const int k0 = base + lane * 8;
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                if ((gc >> h) & 1u) {
                    const float2 l = lc[h];
                    const float eL = __fadd_rn(l.y, __fsub_rn(tp, l.x));  // parity -1
                    const float eR = __fadd_rn(l.x, __fsub_rn(tn, l.y));  // parity +1
                    const unsigned k = static_cast<unsigned>(k0 + h);
                    const unsigned long long kL =
                        (static_cast<unsigned long long>(__float_as_uint(eL)) << 32) | 0x80000000u | k;
                    const unsigned long long kR = (static_cast<unsigned long long>(__float_as_uint(eR)) << 32) | k;
                    best = min(best, min(kL, kR));
                }
            }
#pragma unroll
            for (int h = 0; h < 8; ++h) lc[h] = ln[h];
            gc = gn;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (chainer && lane == 0) pairBest[pr] = best;
        pair_sync(pr);
        if (!chainer && lane == 0) {
            best = min(best, pairBest[pr]);
            // (error bits, featureIdx) of every candidate, for the runner-up report
            candKey[c] = best != ~0ull ? (best & 0xFFFFFFFF00000000ull) | static_cast<unsigned>(f) : ~0ull;
            if (best != ~0ull) {
                refParity[f] = (best & 0x80000000ull) ? int8_t(-1) : int8_t(1);
                refSplit[f] = static_cast<int>(best & 0x7FFFFFFFull);
                atomicMin(&prm->winner, (best & 0xFFFFFFFF00000000ull) | static_cast<unsigned>(f));
            }
        }
        // the pair's buffers, totals and best are reused by its next candidate
        pair_sync(pr);
    }
}

// The replay with the two class chains decoupled, for n <= kRefineSplitMaxN:
// one candidate per CTA.  In a candidate's sorted order the classes come in
// long runs (a good feature separates them), so per-chunk class lists leave
// one chain idle most of the time.  Here the whole order is split first:
//   A. all warps gather every chunk (the sample of each position - its slot
//      mapped back - and its signed weight), keep |w| per position and a
//      bitmask of the positive positions, and count each chunk's positives;
//   B. an exclusive scan of the chunk counts places every position in one of
//      two in-order lists, positives from 0 and negatives from negOff;
//   C. lane 0 of warp 0 adds the positive list and lane 1 the negative list
//      in place, the reference's two sequential FP32 sums (main.cu:626-645),
//      concurrently, 4 addends per 16-byte load, the next load issued ahead;
//      the shorter chain adds +0.0f past its end (no change);
//   D. every position's left sums are its class lists' running sums at its
//      inclusive class ranks, read directly while scoring.
// Inactive samples (+-0 weights) add +0.0f to their class's chain, which
// leaves it unchanged, as in the reference's totals.
constexpr int kRefineSplitMaxN = 26112;  // 8.125 B per position + 64 B of dynamic shared memory

template <bool kTwoCopy>
__global__ void __launch_bounds__(kRefineThreads)
refine_split_kernel(const uint16_t* __restrict__ ord, int64_t ordStride, const uint16_t* __restrict__ gap,
                    int64_t gapStride, const float* __restrict__ wsgG, int n, int slotBase, int L,
                    RoundParams* __restrict__ prm, const int* __restrict__ cand, int8_t* __restrict__ refParity,
                    int* __restrict__ refSplit, unsigned long long* __restrict__ candKey, const int* gate) {
    if (gate_closed(gate)) return;
    const int nc = prm->ncand;
    if (static_cast<int>(blockIdx.x) >= nc) return;
    const int chunks = (n + 255) / 256, nv = chunks * 256;
    extern __shared__ __align__(16) float rsm[];
    float* val = rsm;                                               // [nv] |w| per position
    float* lists = rsm + nv;                                        // [nv + 16] the two class lists
    uint32_t* posMask = reinterpret_cast<uint32_t*>(lists + nv + 16);  // [nv / 32]
    constexpr int kMaxChunks = (kRefineSplitMaxN + 255) / 256;
    __shared__ int chunkPos[kMaxChunks];  // positives before each chunk
    __shared__ int totP, negOff;
    __shared__ unsigned long long warpBest[kRefineWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int f = cand[c];
        const uint16_t* row = ord + static_cast<size_t>(f) * ordStride;
        const uint16_t* grow = gap + static_cast<size_t>(f) * gapStride;
        // A. gather
        for (int i = w; i < chunks; i += kRefineWarps) {
            const int k0 = i * 256 + lane * 8;
            const uint4 v =
                k0 < n ? __ldg(reinterpret_cast<const uint4*>(row + ord_slot(k0, L))) : make_uint4(0, 0, 0, 0);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
            float e[8];
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                uint32_t id = (w4[h >> 1] >> (16 * (h & 1))) & 0xFFFFu;
                if (kTwoCopy) id = slot_sample(id, slotBase);
                e[h] = k0 + h < n ? __ldg(wsgG + id) : 0.0f;
            }
            uint32_t pm = 0;
#pragma unroll
            for (int h = 0; h < 8; ++h)
                if (k0 + h < n && !signbit(e[h])) pm |= 1u << h;
            reinterpret_cast<float4*>(val + k0)[0] = make_float4(fabsf(e[0]), fabsf(e[1]), fabsf(e[2]), fabsf(e[3]));
            reinterpret_cast<float4*>(val + k0)[1] = make_float4(fabsf(e[4]), fabsf(e[5]), fabsf(e[6]), fabsf(e[7]));
            // four lanes' 8-bit masks make one word
            uint32_t word = pm;
            word |= __shfl_down_sync(0xffffffffu, pm, 1) << 8;
            word |= __shfl_down_sync(0xffffffffu, pm, 2) << 16;
            word |= __shfl_down_sync(0xffffffffu, pm, 3) << 24;
            if ((lane & 3) == 0) posMask[i * 8 + (lane >> 2)] = word;
            const int cnt = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(__popc(pm)));
            if (lane == 0) chunkPos[i] = cnt;
        }
        __syncthreads();
        // B. chunk offsets (warp 0), then the two lists
        if (w == 0) {
            int carry = 0;
            for (int i0 = 0; i0 < chunks; i0 += 32) {
                const int x = i0 + lane < chunks ? chunkPos[i0 + lane] : 0;
                int incl = x;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                if (i0 + lane < chunks) chunkPos[i0 + lane] = carry + incl - x;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) {
                totP = carry;
                negOff = (carry + 3) & ~3;
            }
        }
        __syncthreads();
        const int P = totP, N = n - P, nOff = negOff;
        for (int i = w; i < chunks; i += kRefineWarps) {
            const int k0 = i * 256 + lane * 8;
            const uint32_t pm = (posMask[i * 8 + (lane >> 2)] >> (8 * (lane & 3))) & 0xFFu;
            const int mine = __popc(pm);
            int before = mine;  // positives of the chunk before this lane's positions
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, before, o);
                if (lane >= o) before += y;
            }
            before -= mine;
            int rp = chunkPos[i] + before;                        // rank of the next positive
            int rn = (i * 256 - chunkPos[i]) + (lane * 8 - before);  // of the next negative
            const float4 a = reinterpret_cast<const float4*>(val + k0)[0];
            const float4 b = reinterpret_cast<const float4*>(val + k0)[1];
            const float x8[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                if (k0 + h < n) {
                    if ((pm >> h) & 1u)
                        lists[rp++] = x8[h];
                    else
                        lists[nOff + rn++] = x8[h];
                }
            }
        }
        __syncthreads();
        // C. the two chains, concurrently: both lanes over the common length
        // in groups of 4 (the next two groups' loads in flight, the same form
        // as a lone dependent chain), then the longer list alone, then the
        // last addends one by one.  Loads past a list's end stay inside the
        // lists array and are never used.
        if (w == 0 && lane < 2) {
            float* list = lists + (lane == 0 ? 0 : nOff);
            const int mine = lane == 0 ? P : N;
            const int common = min(P, N) & ~3;
            float t = 0.0f;
            auto run = [&](int j, int end) {
                float4 q0 = *reinterpret_cast<const float4*>(list + j);
                float4 q1 = *reinterpret_cast<const float4*>(list + j + 4);
                for (; j < end; j += 4) {
                    const float4 q2 = *reinterpret_cast<const float4*>(list + j + 8);
                    float4 r;
                    t = __fadd_rn(t, q0.x);
                    r.x = t;
                    t = __fadd_rn(t, q0.y);
                    r.y = t;
                    t = __fadd_rn(t, q0.z);
                    r.z = t;
                    t = __fadd_rn(t, q0.w);
                    r.w = t;
                    *reinterpret_cast<float4*>(list + j) = r;
                    q0 = q1;
                    q1 = q2;
                }
                return j;
            };
            int j = run(0, common);
            j = run(j, mine & ~3);
            for (; j < mine; ++j) {
                t = __fadd_rn(t, list[j]);
                list[j] = t;
            }
        }
        __syncthreads();
        const float TP = P > 0 ? lists[P - 1] : 0.0f;
        const float TN = N > 0 ? lists[nOff + N - 1] : 0.0f;
        // D. scoring: the reference's update rule over the splits in order
        // (lower error replaces; at equal error parity +1 replaces parity -1)
        // picks the lexicographic minimum of (error, parity +1 before -1, split
        // index); errors are >= +0, so the float bits order like the values
        // and the triple packs into one key.  A position's left sums are the
        // running sums at its inclusive class ranks.
        unsigned long long best = ~0ull;
        for (int i = w; i < chunks; i += kRefineWarps) {
            const int k0 = i * 256 + lane * 8;
            const uint32_t pm = (posMask[i * 8 + (lane >> 2)] >> (8 * (lane & 3))) & 0xFFu;
            const int mine = __popc(pm);
            int before = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, before, o);
                if (lane >= o) before += y;
            }
            before -= mine;
            if (k0 >= n - 1) continue;
            const int l = k0 / L, r = k0 - l * L;
            const uint32_t g = (static_cast<uint32_t>(__ldg(grow + (r >> 4) * 32 + l)) >> (r & 15)) & 0xFFu;  // gap_word
            int cp = chunkPos[i] + before, cn = (i * 256 - chunkPos[i]) + (lane * 8 - before);
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                if ((pm >> h) & 1u)
                    ++cp;
                else
                    ++cn;
                if ((g >> h) & 1u) {
                    const float lp = cp > 0 ? lists[cp - 1] : 0.0f;
                    const float ln = cn > 0 ? lists[nOff + cn - 1] : 0.0f;
                    const float eL = __fadd_rn(ln, __fsub_rn(TP, lp));  // parity -1
                    const float eR = __fadd_rn(lp, __fsub_rn(TN, ln));  // parity +1
                    const unsigned kk = static_cast<unsigned>(k0 + h);
                    const unsigned long long kL =
                        (static_cast<unsigned long long>(__float_as_uint(eL)) << 32) | 0x80000000u | kk;
                    const unsigned long long kR = (static_cast<unsigned long long>(__float_as_uint(eR)) << 32) | kk;
                    best = min(best, min(kL, kR));
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (lane == 0) warpBest[w] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < kRefineWarps; ++k) best = min(best, warpBest[k]);
            // (error bits, featureIdx) of every candidate, for the runner-up report
            candKey[c] = best != ~0ull ? (best & 0xFFFFFFFF00000000ull) | static_cast<unsigned>(f) : ~0ull;
            if (best != ~0ull) {
                refParity[f] = (best & 0x80000000ull) ? int8_t(-1) : int8_t(1);
                refSplit[f] = static_cast<int>(best & 0x7FFFFFFFull);
                atomicMin(&prm->winner, (best & 0xFFFFFFFF00000000ull) | static_cast<unsigned>(f));
            }
        }
        // the lists and masks are reused by the CTA's next candidate
        __syncthreads();
    }
}

// 5. Winner -> TileBestCandidate with theta = 0.5f * (v[k] + v[k+1]).
// feats and the candidate indices are relative to the searched range, which
// starts at featBase of the pool; the output featureIdx is the pool's.
__global__ void finalize_kernel(const vj_haar_feature* __restrict__ feats, int featBase,
                                const uint32_t* __restrict__ sumT,
                                const float* __restrict__ invNorm, int n, const uint16_t* __restrict__ ord,
                                int64_t ordStride, int slotBase, int L, RoundParams* __restrict__ prm,
                                const int8_t* __restrict__ refParity, const int* __restrict__ refSplit,
                                vj_tile_best* __restrict__ out, const int* gate) {
    if (gate_closed(gate)) return;
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    vj_tile_best b;
    b.pad0 = b.pad1 = b.pad2 = 0;
    const unsigned long long w = prm->winner;
    if (w == ~0ull) {
        b.bestErr = INFINITY;
        b.bestTheta = 0.0f;
        b.featureIdx = -1;
        b.bestParity = 1;
        prm->status = 1;
    } else {
        const int f = static_cast<int>(w & 0xFFFFFFFFull);
        const int k = refSplit[f];
        const uint16_t* row = ord + static_cast<size_t>(f) * ordStride;
        const int s0 = slot_sample(row[ord_slot(k, L)], slotBase), s1 = slot_sample(row[ord_slot(k + 1, L)], slotBase);
        const vj_haar_feature ft = feats[f];
        const float v0 = train_response(ft, sumT, n, s0, invNorm[s0]);
        const float v1 = train_response(ft, sumT, n, s1, invNorm[s1]);
        b.bestErr = __uint_as_float(static_cast<uint32_t>(w >> 32));
        b.bestTheta = __fmul_rn(0.5f, __fadd_rn(v0, v1));
        b.featureIdx = featBase + f;
        b.bestParity = refParity[f];
    }
    *out = b;
}

// ReduceTileBestCandidatesKernel (main.cu:991-1028): the best of n tile (or
// rank) candidates, lower FP32 error first, then lower featureIdx; one warp.
__device__ __forceinline__ vj_tile_best better_tile(const vj_tile_best& a, const vj_tile_best& b) {
    if (b.bestErr < a.bestErr) return b;
    if (b.bestErr > a.bestErr) return a;
    return b.featureIdx < a.featureIdx ? b : a;
}

__global__ void reduce_tile_best_kernel(const vj_tile_best* __restrict__ in, int n, vj_tile_best* __restrict__ out) {
    vj_tile_best best;
    best.bestErr = INFINITY;
    best.bestTheta = 0.0f;
    best.featureIdx = INT_MAX;
    best.bestParity = 1;
    best.pad0 = best.pad1 = best.pad2 = 0;
    for (int i = threadIdx.x; i < n; i += 32) best = better_tile(best, in[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vj_tile_best other = best;
        other.bestErr = __shfl_xor_sync(0xffffffffu, best.bestErr, o);
        other.bestTheta = __shfl_xor_sync(0xffffffffu, best.bestTheta, o);
        other.featureIdx = __shfl_xor_sync(0xffffffffu, best.featureIdx, o);
        other.bestParity = static_cast<int8_t>(__shfl_xor_sync(0xffffffffu, static_cast<int>(best.bestParity), o));
        best = better_tile(best, other);
    }
    if (threadIdx.x == 0) *out = best;
}

// ---------------------------------------------------------------------------
// AdaBoost round update (main.cu:2082-2166, kernels main.cu:829-906) with FP64
// alpha/log and renormalisation, in two kernels with the arithmetic of one
// 1024-thread block: partial t of 1024 is the double sum, in sample order, of
// the new unnormalised weights of samples t, t+1024, ...; the normaliser Z is
// the halving-tree sum of the 1024 partials, and every weight is divided by Z
// in double, so the result does not depend on scheduling.  The first kernel
// computes every sample's new weight on its own thread (ceil(n / 1024) blocks
// of 1024), and the last block to finish adds the partials in that order, one
// per thread; the second spreads the divisions (FP64) over many blocks, each
// rebuilding Z from the partials in the same tree order.
// ---------------------------------------------------------------------------
constexpr int kRoundPartials = 1024;

__device__ __forceinline__ bool best_valid(const vj_tile_best& b) { return b.featureIdx >= 0 && isfinite(b.bestErr); }

__global__ void __launch_bounds__(1024, 1)
round_update_kernel(const vj_haar_feature* __restrict__ feats, const vj_tile_best* __restrict__ best,
                    const uint32_t* __restrict__ sumT, const float* __restrict__ invNorm,
                    const int8_t* __restrict__ label, const uint8_t* __restrict__ active,
                    const float* __restrict__ weight, float* __restrict__ strong, int n,
                    uint8_t* __restrict__ usedMask, vj_weak_classifier* __restrict__ weakOut,
                    int* __restrict__ status, double* __restrict__ xbuf, double* __restrict__ partials,
                    PruneState* __restrict__ ps, int* gate, unsigned int* __restrict__ done) {
    if (gate_closed(gate)) return;
    __shared__ vj_haar_feature sfeat;
    __shared__ float sTheta, sLeft, sRight;
    __shared__ double sF;
    __shared__ int sPar, sValid;
    __shared__ bool lastBlock;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // sample
    if (threadIdx.x == 0) {
        const vj_tile_best b = *best;
        const bool valid = best_valid(b);
        sValid = valid ? 1 : 0;
        if (valid) {
            const float eps = 1e-6f;
            const float e = fminf(fmaxf(b.bestErr, eps), __fsub_rn(1.0f, eps));
            const double ed = static_cast<double>(e);
            const float C = static_cast<float>(log((1.0 - ed) / ed));
            sF = exp(static_cast<double>(C));
            if (ps && blockIdx.x == 0) ps->F = sF;
            sTheta = b.bestTheta;
            sPar = b.bestParity;
            sLeft = b.bestParity > 0 ? -C : C;
            sRight = b.bestParity > 0 ? C : -C;
            sfeat = feats[b.featureIdx];
            if (blockIdx.x == 0) {
                if (weakOut) {
                    vj_weak_classifier wc;
                    wc.featureIdx = b.featureIdx;
                    wc.theta = b.bestTheta;
                    wc.parity = b.bestParity;
                    wc.pad0 = wc.pad1 = wc.pad2 = 0;
                    wc.err = e;
                    wc.alpha = C;
                    wc.leftVal = sLeft;
                    wc.rightVal = sRight;
                    *weakOut = wc;
                }
                if (usedMask) usedMask[b.featureIdx] = 1;
            }
        }
        if (blockIdx.x == 0) {
            if (status) *status = valid ? 0 : 1;
            if (!valid && gate) *gate = 2;
        }
    }
    __syncthreads();
    if (!sValid) return;
    const vj_haar_feature f = sfeat;
    const float theta = sTheta, left = sLeft, right = sRight;
    const double F = sF;
    const int par = sPar;
    if (i < n) {
        const float r = train_response(f, sumT, n, i, invNorm[i]);
        const bool lt = r < theta;
        strong[i] = __fadd_rn(strong[i], lt ? left : right);
        double x = 0.0;
        if (active == nullptr || active[i] != 0) {
            const int pred = par > 0 ? (lt ? -1 : 1) : (lt ? 1 : -1);
            x = static_cast<double>(weight[i]);
            if (pred != label[i]) x = x * F;
        }
        xbuf[i] = x;
    }
    __threadfence();  // this block's xbuf before its count
    __syncthreads();
    if (threadIdx.x == 0) lastBlock = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!lastBlock) return;
    // partial t: samples t, t+1024, ... in order (an inactive sample's +0.0
    // leaves the sum as it is), eight loads in flight per step
    __threadfence();
    for (int t = threadIdx.x; t < kRoundPartials; t += blockDim.x) {
        double acc = 0.0;
        for (int i0 = t; i0 < n; i0 += 8 * kRoundPartials) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = i0 + u * kRoundPartials < n ? __ldcg(xbuf + i0 + u * kRoundPartials) : 0.0;
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (i0 + u * kRoundPartials < n) acc += v[u];
        }
        partials[t] = acc;
    }
    if (threadIdx.x == 0) *done = 0u;  // ready for the next launch
}

// With wShadow given, the new weights are also written there, and block 0
// records the factor that takes a feature's exact error under the old weights
// to a lower bound under the new ones: every new weight is at least
// min(1, F) / Z times the old one, up to the FP32 rounding of the division
// (relative 2^-24, covered by the factor 1 - 4u).
__global__ void __launch_bounds__(256)
round_normalize_kernel(const vj_tile_best* __restrict__ best, const double* __restrict__ xbuf,
                       const double* __restrict__ partials, float* __restrict__ weight, int n,
                       float* __restrict__ wShadow, PruneState* __restrict__ ps, const int* gate) {
    if (gate_closed(gate)) return;
    if (!best_valid(*best)) return;
    __shared__ double part[kRoundPartials];
    for (int k = threadIdx.x; k < kRoundPartials; k += blockDim.x) part[k] = partials[k];
    __syncthreads();
    for (int s = kRoundPartials / 2; s >= 1; s >>= 1) {
        for (int k = threadIdx.x; k < s; k += blockDim.x) part[k] = part[k] + part[k + s];
        __syncthreads();
    }
    const double Z = part[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = xbuf[i];
        const float w = (Z > 1e-30) ? static_cast<float>(x / Z) : static_cast<float>(x);
        weight[i] = w;
        if (wShadow) wShadow[i] = w;
    }
    if (ps && blockIdx.x == 0 && threadIdx.x == 0) {
        const double u = 5.9604644775390625e-08;
        const double g = (Z > 1e-30) ? fmin(1.0, ps->F) / Z * (1.0 - 4.0 * u) : 0.0;
        ps->scale = __double2float_rd(fmin(g, 1.0));
        ps->valid = g > 0.0 ? 1 : 0;
    }
}

// Stage calibration (main.cu:2168-2300) in one CTA: radix select of the
// cutIdx-th smallest positive score in DeviceRadixSort order, then the four
// counts of CountPassAndNegKernel (main.cu:935-958).
__global__ void __launch_bounds__(1024)
stage_calib_kernel(const float* __restrict__ strong, const uint8_t* __restrict__ active, int n,
                   int numPos, float minHitRate, float maxFalseAlarm, int stageNegBase,
                   vj_stage_calib* __restrict__ out, int* gate) {
    if (gate_closed(gate)) return;
    __shared__ uint32_t hist[256];
    __shared__ uint32_t sPrefix, sK;
    __shared__ int cnt[4];
    const int tid = threadIdx.x;
    const int need = static_cast<int>(ceilf(__fmul_rn(minHitRate, static_cast<float>(numPos))));
    const int minPass = need > 1 ? need : 1;
    const int cutIdx = numPos - minPass;
    if (tid == 0) {
        sPrefix = 0;
        sK = static_cast<uint32_t>(cutIdx < 0 ? 0 : cutIdx);
    }
    __syncthreads();
    for (int pass = 3; pass >= 0; --pass) {
        const int shift = pass * 8;
        for (int i = tid; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = sPrefix;
        const uint32_t himask = pass == 3 ? 0u : (0xFFFFFFFFu << (shift + 8));
        for (int i = tid; i < numPos; i += blockDim.x) {
            const uint32_t k = radix_key(__float_as_uint(strong[i]));
            if ((k & himask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        // The digit: the first d < 255 whose inclusive count C(d) exceeds
        // the rank k (else 255), and the rank within it k - C(d - 1).  Warp
        // 0 scans the 256 counts, 8 consecutive digits per lane.
        if (tid < 32) {
            const uint32_t kk = sK;
            uint32_t h[8], sum = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                h[j] = hist[tid * 8 + j];
                sum += h[j];
            }
            uint32_t incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += y;
            }
            const unsigned over = __ballot_sync(0xffffffffu, incl > kk);
            const int lane = over ? __ffs(over) - 1 : 31;
            if (tid == lane) {
                uint32_t run = incl - sum, d = static_cast<uint32_t>(tid * 8);
                int j = 0;
                while (j < 7 && d < 255u && run + h[j] <= kk) {
                    run += h[j];
                    ++d;
                    ++j;
                }
                if (d < 255u && run + h[j] <= kk) {  // lane 31 past its last digit: capped at 255
                    run += h[j];
                    ++d;
                }
                sK = kk - run;
                sPrefix = prefix | (d << shift);
            }
        }
        __syncthreads();
    }
    const uint32_t kb = sPrefix;
    const uint32_t bits = (kb & 0x80000000u) ? (kb ^ 0x80000000u) : ~kb;
    const float cut = __uint_as_float(bits);
    if (tid < 4) cnt[tid] = 0;
    __syncthreads();
    int pge = 0, pgt = 0, nge = 0, ngt = 0;
    for (int i = tid; i < n; i += blockDim.x) {
        const float s = strong[i];
        if (i < numPos) {
            pge += s >= cut;
            pgt += s > cut;
        } else if (active == nullptr || active[i] != 0) {
            nge += s >= cut;
            ngt += s > cut;
        }
    }
    atomicAdd(&cnt[0], pge);
    atomicAdd(&cnt[1], pgt);
    atomicAdd(&cnt[2], nge);
    atomicAdd(&cnt[3], ngt);
    __syncthreads();
    if (tid == 0) {
        const bool strictGt = cnt[1] >= minPass;
        vj_stage_calib r;
        r.cutVal = cut;
        r.stageThreshold = strictGt ? nextafterf(cut, INFINITY) : cut;
        r.strictGt = strictGt ? 1 : 0;
        r.posPass = strictGt ? cnt[1] : cnt[0];
        r.negSurvive = strictGt ? cnt[3] : cnt[2];
        r.hitRate = __fdiv_rn(static_cast<float>(r.posPass), static_cast<float>(numPos));
        r.falseAlarm = __fdiv_rn(static_cast<float>(r.negSurvive), static_cast<float>(stageNegBase));
        r.satisfied = ((r.hitRate >= minHitRate && r.falseAlarm <= maxFalseAlarm) || r.negSurvive == 0) ? 1 : 0;
        *out = r;
        if (r.satisfied && gate) *gate = 1;
    }
}

// ---------------------------------------------------------------------------
// Reference step API (AdaBoostTrainer members).
// ---------------------------------------------------------------------------
__global__ void eval_responses_kernel(const vj_haar_feature* __restrict__ feats, int featBegin,
                                      int featCount, const uint32_t* __restrict__ sumT,
                                      const float* __restrict__ invNorm, int n, float* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int fl = blockIdx.y;
    if (s >= n || fl >= featCount) return;
    const vj_haar_feature f = feats[featBegin + fl];
    out[static_cast<size_t>(fl) * n + s] = train_response(f, sumT, n, s, __ldg(invNorm + s));
}

struct SplitBest {
    float err;
    int split;
    int parity;
};

// betterBest, boosting_core.cu:59-79: err, then smaller split, then parity +1.
__device__ __forceinline__ SplitBest better(const SplitBest& a, const SplitBest& b) {
    if (b.err < a.err) return b;
    if (b.err > a.err) return a;
    if (b.split < a.split) return b;
    if (b.split > a.split) return a;
    return b.parity > a.parity ? b : a;
}

// EvaluateAndFindThresholdKernel (boosting_core.cu:289-456) semantics with the
// prefix sums of sweep_kernel; one warp per feature.
__global__ void __launch_bounds__(256)
find_thresholds_kernel(const float* __restrict__ resp, const uint16_t* __restrict__ sorted, int n,
                       int featCount, const float* __restrict__ wsg, const RoundParams* __restrict__ prm,
                       vj_feature_best_split* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (f >= featCount) return;
    const float* rrow = resp + static_cast<size_t>(f) * n;
    const uint16_t* orow = sorted + static_cast<size_t>(f) * n;
    const float TP = prm->tp, TN = prm->tn;
    SplitBest best{FLT_MAX, -1, 1};
    float cp = 0.0f, cn = 0.0f, kp = 0.0f, kn = 0.0f;
    for (int base = 0; base < n - 1; base += 256) {
        const int k0 = base + lane * 8;
        float lp[8], ln[8];
        bool ok[8];
        float sp = 0.0f, sn = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int k = k0 + i;
            float x = 0.0f;
            ok[i] = false;
            if (k < n) {
                const int s = orow[k];
                x = wsg[s];
                if (k + 1 < n) ok[i] = __fadd_rn(rrow[s], 1e-7f) < rrow[orow[k + 1]];
            }
            sp = __fadd_rn(sp, fmaxf(x, 0.0f));
            sn = __fadd_rn(sn, fmaxf(-x, 0.0f));
            lp[i] = sp;
            ln[i] = sn;
        }
        float ip = sp, in = sn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float yp = __shfl_up_sync(0xffffffffu, ip, o);
            const float yn = __shfl_up_sync(0xffffffffu, in, o);
            if (lane >= o) {
                ip = __fadd_rn(ip, yp);
                in = __fadd_rn(in, yn);
            }
        }
        float ep = __shfl_up_sync(0xffffffffu, ip, 1), en = __shfl_up_sync(0xffffffffu, in, 1);
        if (lane == 0) ep = en = 0.0f;
        const float totp = __shfl_sync(0xffffffffu, ip, 31), totn = __shfl_sync(0xffffffffu, in, 31);
        const float bp = __fadd_rn(cp, ep), bn = __fadd_rn(cn, en);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (ok[i]) {
                const float Lp = __fadd_rn(bp, lp[i]), Ln = __fadd_rn(bn, ln[i]);
                const float eP = __fadd_rn(Ln, __fsub_rn(TP, Lp));
                const float eN = __fadd_rn(Lp, __fsub_rn(TN, Ln));
                best = better(best, SplitBest{eP, k0 + i, -1});
                best = better(best, SplitBest{eN, k0 + i, 1});
            }
        }
        {
            const float y = __fsub_rn(totp, kp), t = __fadd_rn(cp, y);
            kp = __fsub_rn(__fsub_rn(t, cp), y);
            cp = t;
        }
        {
            const float y = __fsub_rn(totn, kn), t = __fadd_rn(cn, y);
            kn = __fsub_rn(__fsub_rn(t, cn), y);
            cn = t;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        SplitBest other{__shfl_xor_sync(0xffffffffu, best.err, o), __shfl_xor_sync(0xffffffffu, best.split, o),
                        __shfl_xor_sync(0xffffffffu, best.parity, o)};
        best = better(best, other);
    }
    if (lane == 0) {
        vj_feature_best_split r;
        r.pad0 = r.pad1 = r.pad2 = 0;
        if (best.split >= 0 && best.split < n - 1) {
            r.bestErr = best.err;
            r.bestSplitPos = best.split;
            r.bestParity = static_cast<int8_t>(best.parity);
            r.bestTheta = __fmul_rn(0.5f, __fadd_rn(rrow[orow[best.split]], rrow[orow[best.split + 1]]));
        } else {
            r.bestErr = FLT_MAX;
            r.bestSplitPos = best.split;
            r.bestParity = 1;
            r.bestTheta = 0.0f;
        }
        out[f] = r;
    }
}

// SelectBestInTileKernel (boosting_core.cu:155-192): err, then lower featureIdx.
__global__ void __launch_bounds__(256)
select_tile_kernel(const vj_feature_best_split* __restrict__ best, int featBegin, int featCount,
                   const uint8_t* __restrict__ usedMask, vj_tile_best* __restrict__ out) {
    __shared__ float se[256];
    __shared__ int sf[256];
    __shared__ float st[256];
    __shared__ int sp[256];
    float e = FLT_MAX, th = 0.0f;
    int fi = INT_MAX, par = 1;
    for (int i = threadIdx.x; i < featCount; i += blockDim.x) {
        const int g = featBegin + i;
        if (usedMask && usedMask[g]) continue;
        const vj_feature_best_split b = best[i];
        if (b.bestErr < e || (b.bestErr == e && g < fi)) {
            e = b.bestErr;
            th = b.bestTheta;
            fi = g;
            par = b.bestParity;
        }
    }
    se[threadIdx.x] = e;
    sf[threadIdx.x] = fi;
    st[threadIdx.x] = th;
    sp[threadIdx.x] = par;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            const int o = threadIdx.x + s;
            if (se[o] < se[threadIdx.x] || (se[o] == se[threadIdx.x] && sf[o] < sf[threadIdx.x])) {
                se[threadIdx.x] = se[o];
                sf[threadIdx.x] = sf[o];
                st[threadIdx.x] = st[o];
                sp[threadIdx.x] = sp[o];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        vj_tile_best r;
        r.bestErr = se[0];
        r.bestTheta = st[0];
        r.featureIdx = sf[0];
        r.bestParity = static_cast<int8_t>(sp[0]);
        r.pad0 = r.pad1 = r.pad2 = 0;
        *out = r;
    }
}

int sm_count() {
    static int cached = 0;
    if (!cached) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached = v > 0 ? v : 1;
    }
    return cached;
}

// Blocks of the refine launch: one per SM (each warp takes candidates in turn).
int refine_blocks() { return sm_count(); }

// Launches eval_sort_kernel with the smallest items-per-thread that holds n.
// keyScratch / idxScratch: 2 * 1024 * large_sort_r(n) keys and indices per
// CTA of the launch (min(featCount, SMs) CTAs), used only for n > 32768.
int launch_eval_sort(const vj_haar_feature* feats, int featBegin, int featCount, const uint32_t* sumT,
                     const float* invNorm, int n, const float* resp, uint16_t* ordOut, int64_t ordStride,
                     bool ordPadded, uint16_t* gapOut, int64_t gapStride, int slotBase, int L, uint32_t* keyScratch,
                     uint16_t* idxScratch, cudaStream_t stream) {
    const int grid = std::min(featCount, sm_count());
    auto go = [&](auto kernel, size_t smem) -> int {
        VJ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        VJ_TIMED_LAUNCH("eval_sort_kernel", stream,
                        kernel<<<grid, kSortThreads, smem, stream>>>(feats, featBegin, featCount, sumT, invNorm, n,
                                                                     resp, ordOut, ordStride, ordPadded, gapOut,
                                                                     gapStride, slotBase, L));
        VJ_LAUNCH_CHECK("eval_sort_kernel");
        return VJ_OK;
    };
#define VJ_SORT_CASE(RR)                                                                   \
    if (n <= 1024 * RR)                                                                    \
        return resp ? go(eval_sort_kernel<RR, true>, sort_smem_bytes<RR>())                \
                    : go(eval_sort_kernel<RR, false>, sort_smem_bytes<RR>());
    VJ_SORT_CASE(4)
    VJ_SORT_CASE(8)
    VJ_SORT_CASE(16)
    if (n <= 1024 * kBlockedMaxR)
        return resp ? go(eval_sort_blocked_kernel<kBlockedMaxR, true>, blocked_sort_smem_bytes<kBlockedMaxR>())
                    : go(eval_sort_blocked_kernel<kBlockedMaxR, false>, blocked_sort_smem_bytes<kBlockedMaxR>());
    VJ_SORT_CASE(24)
    VJ_SORT_CASE(32)
#undef VJ_SORT_CASE
    const int R = large_sort_r(n);
    if (R > kLargeSortMaxR) return set_error(VJ_INVALID_ARG, "the sort holds at most 65535 samples per feature");
    if (!keyScratch || !idxScratch) return set_error(VJ_RUNTIME_ERROR, "sort: no scratch for more than 32768 samples");
    auto kernel = resp ? eval_sort_large_kernel<true> : eval_sort_large_kernel<false>;
    const size_t smem = large_sort_smem_bytes(R);
    VJ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    VJ_TIMED_LAUNCH("eval_sort_kernel", stream,
                    kernel<<<grid, kSortThreads, smem, stream>>>(feats, featBegin, featCount, sumT, invNorm, n, resp,
                                                                 ordOut, ordStride, ordPadded, gapOut, gapStride, L, R,
                                                                 keyScratch, idxScratch));
    VJ_LAUNCH_CHECK("eval_sort_large_kernel");
    return VJ_OK;
}

}  // namespace
}  // namespace vjgb

using namespace vjgb;

struct vj_trainer {
    int winW = 24, winH = 24, maxSamples = 0;
    vj_haar_feature* d_feat = nullptr;
    int64_t nFeat = 0;
    // Features searched by vj_stump_search: [rangeBegin, rangeBegin + rangeCount)
    // of the pool (rangeCount < 0: the whole pool).
    int64_t rangeBegin = 0, rangeCount = -1;
    const uint32_t* d_sumT = nullptr;
    const float* d_invNorm = nullptr;
    int n = 0;
    const int8_t* d_label = nullptr;
    const uint8_t* d_active = nullptr;
    float* d_weight = nullptr;
    // Per-feature sample orders and valid-split masks.
    uint16_t* d_ord = nullptr;
    uint16_t* d_gap = nullptr;
    size_t ordBytes = 0, gapBytes = 0;
    int64_t ordStride = 0, gapStride = 0;
    int slotBase = 0;  // > 0: resident orders hold two-copy shared-memory slots
    int laneRun = 16;  // L of the resident layout (lane_run(n))
    bool prepared = false;
    // Keys and indices of the sort above 32,768 samples (per CTA of the launch).
    uint32_t* d_sortKeys = nullptr;
    uint16_t* d_sortIdx = nullptr;
    size_t sortScratchPositions = 0;
    // Per-round scratch.
    float* d_wsg = nullptr;
    float* d_fastErr = nullptr;
    int* d_cand = nullptr;
    unsigned long long* d_candKey = nullptr;
    double* d_xbuf = nullptr;      // unnormalised new weights of the round update
    double* d_partials = nullptr;  // its 1024 partial sums
    float2* d_prefix = nullptr;    // refine: left sums after each position, one row per warp
    int8_t* d_refParity = nullptr;
    int* d_refSplit = nullptr;
    RoundParams* d_prm = nullptr;
    PrepPartial* d_prepPart = nullptr;  // prep_round_kernel's per-block totals
    unsigned int* d_prepDone = nullptr; // its count of finished blocks (0 between launches)
    unsigned int* d_updDone = nullptr;  // round_update_kernel's count of finished blocks
    int* d_status = nullptr;
    // Sweep pruning: per-feature lower bounds of the exact best error, the
    // weights as the last round update left them, the active mask as the last
    // search saw it, and the last update's factor; reset (no pruning in the
    // next search) whenever the training set, the pool or the range changes.
    float* d_lb = nullptr;
    float* d_wShadow = nullptr;
    uint8_t* d_aShadow = nullptr;
    PruneState* d_prune = nullptr;
    bool pruneReset = true;
    unsigned long long* d_sweptTotal = nullptr;  // features streamed since the trainer was created
    int* d_gate = nullptr;  // stage gate of the round kernels (caller's memory), or none
    int64_t scratchFeat = 0;
    int scratchN = 0;
};

namespace {

int ensure_round_scratch(vj_trainer* t) {
    if (t->scratchFeat >= t->nFeat && t->scratchN >= t->n && t->d_prm) return VJ_OK;
    cudaFree(t->d_wsg);
    cudaFree(t->d_fastErr);
    cudaFree(t->d_cand);
    cudaFree(t->d_candKey);
    cudaFree(t->d_xbuf);
    cudaFree(t->d_partials);
    cudaFree(t->d_prefix);
    cudaFree(t->d_refParity);
    cudaFree(t->d_refSplit);
    cudaFree(t->d_lb);
    cudaFree(t->d_wShadow);
    cudaFree(t->d_aShadow);
    t->d_lb = t->d_wShadow = nullptr;
    t->d_aShadow = nullptr;
    t->d_wsg = nullptr;
    t->d_fastErr = nullptr;
    t->d_cand = nullptr;
    t->d_candKey = nullptr;
    t->d_xbuf = nullptr;
    t->d_partials = nullptr;
    t->d_prefix = nullptr;
    t->d_refParity = nullptr;
    t->d_refSplit = nullptr;
    t->scratchFeat = t->scratchN = 0;
    const int64_t F = t->nFeat > 0 ? t->nFeat : 1;
    const int N = t->maxSamples;
    VJ_CUDA_TRY(cudaMalloc(&t->d_wsg, sizeof(float) * (N + 1)));  // + the zero slot at n
    VJ_CUDA_TRY(cudaMalloc(&t->d_fastErr, sizeof(float) * F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_cand, sizeof(int) * F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_candKey, sizeof(unsigned long long) * F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_xbuf, sizeof(double) * N));
    VJ_CUDA_TRY(cudaMalloc(&t->d_partials, sizeof(double) * kRoundPartials));
    VJ_CUDA_TRY(cudaMalloc(&t->d_prefix, sizeof(float2) * static_cast<size_t>(refine_blocks()) * kRefineWarps * N));
    VJ_CUDA_TRY(cudaMalloc(&t->d_refParity, F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_refSplit, sizeof(int) * F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_lb, sizeof(float) * F));
    VJ_CUDA_TRY(cudaMalloc(&t->d_wShadow, sizeof(float) * N));
    VJ_CUDA_TRY(cudaMalloc(&t->d_aShadow, N));
    if (!t->d_prune) VJ_CUDA_TRY(cudaMalloc(&t->d_prune, sizeof(PruneState)));
    if (!t->d_sweptTotal) {
        VJ_CUDA_TRY(cudaMalloc(&t->d_sweptTotal, sizeof(unsigned long long)));
        VJ_CUDA_TRY(cudaMemset(t->d_sweptTotal, 0, sizeof(unsigned long long)));
    }
    t->pruneReset = true;
    if (!t->d_prm) VJ_CUDA_TRY(cudaMalloc(&t->d_prm, sizeof(RoundParams)));
    if (!t->d_prepPart) {
        VJ_CUDA_TRY(cudaMalloc(&t->d_prepPart, sizeof(PrepPartial) * kPrepMaxBlocks));
        VJ_CUDA_TRY(cudaMalloc(&t->d_prepDone, sizeof(unsigned int)));
        VJ_CUDA_TRY(cudaMemset(t->d_prepDone, 0, sizeof(unsigned int)));
        VJ_CUDA_TRY(cudaMalloc(&t->d_updDone, sizeof(unsigned int)));
        VJ_CUDA_TRY(cudaMemset(t->d_updDone, 0, sizeof(unsigned int)));
    }
    if (!t->d_status) VJ_CUDA_TRY(cudaMalloc(&t->d_status, sizeof(int)));
    t->scratchFeat = F;
    t->scratchN = N;
    return VJ_OK;
}

// The global scratch of the sort for n > 32768: two key and two index
// buffers of 1024 * large_sort_r(n) positions for each CTA (one per SM).
int ensure_sort_scratch(vj_trainer* t, int n) {
    if (n <= kOnChipSortMax) return VJ_OK;
    const size_t positions = static_cast<size_t>(sm_count()) * 2 * 1024 * large_sort_r(n);
    if (positions <= t->sortScratchPositions) return VJ_OK;
    cudaFree(t->d_sortKeys);
    cudaFree(t->d_sortIdx);
    t->d_sortKeys = nullptr;
    t->d_sortIdx = nullptr;
    t->sortScratchPositions = 0;
    VJ_CUDA_TRY(cudaMalloc(&t->d_sortKeys, positions * sizeof(uint32_t)));
    VJ_CUDA_TRY(cudaMalloc(&t->d_sortIdx, positions * sizeof(uint16_t)));
    t->sortScratchPositions = positions;
    return VJ_OK;
}

int64_t range_begin(const vj_trainer* t) { return t->rangeCount < 0 ? 0 : t->rangeBegin; }
int64_t range_count(const vj_trainer* t) { return t->rangeCount < 0 ? t->nFeat : t->rangeCount; }

int check_bound(vj_trainer* t, const char* fn) {
    if (!t) return set_error(VJ_INVALID_ARG, std::string(fn) + ": null trainer");
    if (!t->d_feat || t->nFeat <= 0) return set_error(VJ_INVALID_ARG, std::string(fn) + ": no feature pool set");
    if (!t->d_sumT || t->n <= 0) return set_error(VJ_INVALID_ARG, std::string(fn) + ": no training set bound");
    return VJ_OK;
}

// Writes the per-feature orders and split masks for the whole pool.
int sort_all(vj_trainer* t, cudaStream_t s) {
    const int L = lane_run(t->n);
    const int64_t ordStride = 32 * static_cast<int64_t>(L);  // 32 lane runs
    const int64_t gapStride = 2 * static_cast<int64_t>(L);   // 16-bit words
    const int64_t F = range_count(t);
    const size_t ordBytes = static_cast<size_t>(F) * ordStride * sizeof(uint16_t);
    const size_t gapBytes = static_cast<size_t>(F) * gapStride * sizeof(uint16_t);
    if (ordBytes > t->ordBytes) {
        cudaFree(t->d_ord);
        t->d_ord = nullptr;
        t->ordBytes = 0;
        VJ_CUDA_TRY(cudaMalloc(&t->d_ord, ordBytes));
        t->ordBytes = ordBytes;
    }
    if (gapBytes > t->gapBytes) {
        cudaFree(t->d_gap);
        t->d_gap = nullptr;
        t->gapBytes = 0;
        VJ_CUDA_TRY(cudaMalloc(&t->d_gap, gapBytes));
        t->gapBytes = gapBytes;
    }
    t->ordStride = ordStride;
    t->gapStride = gapStride;
    t->slotBase = t->n <= kTwoCopyMax ? two_copy_base(t->n) : 0;
    t->laneRun = L;
    const int st = ensure_sort_scratch(t, t->n);
    if (st != VJ_OK) return st;
    return launch_eval_sort(t->d_feat, static_cast<int>(range_begin(t)), static_cast<int>(F), t->d_sumT,
                            t->d_invNorm, t->n, nullptr,
                            t->d_ord, ordStride, true, t->d_gap, gapStride, t->slotBase, L, t->d_sortKeys,
                            t->d_sortIdx, s);
}

}  // namespace

extern "C" {

int vj_trainer_create(int winW, int winH, int maxSamples, vj_trainer** out) {
    if (!out) return set_error(VJ_INVALID_ARG, "vj_trainer_create: null out");
    *out = nullptr;
    if (winW != kWin || winH != kWin)
        return set_error(VJ_INVALID_ARG, "vj_trainer_create: the training window is 24x24");
    if (maxSamples <= 1 || maxSamples > kMaxSamples)
        return set_error(VJ_INVALID_ARG, "vj_trainer_create: maxSamples must be in [2, 65535]");
    auto* t = new vj_trainer();
    t->winW = winW;
    t->winH = winH;
    t->maxSamples = maxSamples;
    *out = t;
    return ok();
}

int vj_trainer_destroy(vj_trainer* t) {
    if (!t) return ok();
    cudaFree(t->d_feat);
    cudaFree(t->d_ord);
    cudaFree(t->d_gap);
    cudaFree(t->d_wsg);
    cudaFree(t->d_fastErr);
    cudaFree(t->d_cand);
    cudaFree(t->d_candKey);
    cudaFree(t->d_xbuf);
    cudaFree(t->d_partials);
    cudaFree(t->d_prefix);
    cudaFree(t->d_refParity);
    cudaFree(t->d_refSplit);
    cudaFree(t->d_prm);
    cudaFree(t->d_prepPart);
    cudaFree(t->d_prepDone);
    cudaFree(t->d_updDone);
    cudaFree(t->d_status);
    cudaFree(t->d_sortKeys);
    cudaFree(t->d_sortIdx);
    cudaFree(t->d_lb);
    cudaFree(t->d_wShadow);
    cudaFree(t->d_aShadow);
    cudaFree(t->d_prune);
    cudaFree(t->d_sweptTotal);
    delete t;
    return ok();
}

int vj_trainer_set_features(vj_trainer* t, const vj_haar_feature* features, int64_t count) {
    if (!t || !features || count <= 0 || count > INT_MAX)
        return set_error(VJ_INVALID_ARG, "vj_trainer_set_features: bad arguments");
    for (int64_t i = 0; i < count; ++i) {
        const vj_haar_feature& f = features[i];
        const vj_fast_rect* rr[3] = {&f.r0, &f.r1, &f.r2};
        // Tilted features train like the reference trains them: their four
        // corner indices are read from the upright integral like any others
        // (the reference builds no tilted integral; IntegralImageSetT::d_tiltedT
        // stays null, face_vision_engine.cu:1171).
        if (f.rectCount != 2 && f.rectCount != 3)
            return set_error(VJ_INVALID_ARG, "vj_trainer_set_features: features have 2 or 3 rectangles");
        for (int r = 0; r < f.rectCount; ++r) {
            const int32_t p[4] = {rr[r]->p0, rr[r]->p1, rr[r]->p2, rr[r]->p3};
            for (int c = 0; c < 4; ++c)
                if (p[c] < 0 || p[c] >= kIIArea)
                    return set_error(VJ_INVALID_ARG, "vj_trainer_set_features: corner outside the 25x25 integral");
        }
    }
    cudaFree(t->d_feat);
    t->d_feat = nullptr;
    t->nFeat = 0;
    t->rangeBegin = 0;
    t->rangeCount = -1;
    t->prepared = false;
    t->pruneReset = true;
    VJ_CUDA_TRY(cudaMalloc(&t->d_feat, sizeof(vj_haar_feature) * count));
    VJ_CUDA_TRY(cudaMemcpy(t->d_feat, features, sizeof(vj_haar_feature) * count, cudaMemcpyHostToDevice));
    t->nFeat = count;
    return ok();
}

int vj_trainer_bind(vj_trainer* t, const uint32_t* d_sumT, const float* d_invNorm, int n,
                    const int8_t* d_label, const uint8_t* d_active, float* d_weight) {
    if (!t || !d_sumT || !d_invNorm || !d_label || !d_weight)
        return set_error(VJ_INVALID_ARG, "vj_trainer_bind: null view");
    if (n <= 1 || n > t->maxSamples)
        return set_error(VJ_INVALID_ARG, "vj_trainer_bind: sample count outside [2, maxSamples]");
    t->d_sumT = d_sumT;
    t->d_invNorm = d_invNorm;
    t->n = n;
    t->d_label = d_label;
    t->d_active = d_active;
    t->d_weight = d_weight;
    t->prepared = false;
    t->pruneReset = true;
    return ok();
}

int vj_trainer_last_round(vj_trainer* t, vj_round_info* out) {
    if (!t || !out || !t->d_prm) return set_error(VJ_INVALID_ARG, "vj_trainer_last_round: no search has run");
    RoundParams p;
    VJ_CUDA_TRY(cudaDeviceSynchronize());
    VJ_CUDA_TRY(cudaMemcpy(&p, t->d_prm, sizeof(p), cudaMemcpyDeviceToHost));
    out->fastMin = bits_float(static_cast<int32_t>(p.fastMinBits));
    out->window = p.window;
    out->candidates = p.ncand;
    out->status = p.status;
    out->totalPos = p.tp;
    out->totalNeg = p.tn;
    out->swept = p.swept;
    out->pad0 = 0;
    unsigned long long total = 0;
    VJ_CUDA_TRY(cudaMemcpy(&total, t->d_sweptTotal, sizeof(total), cudaMemcpyDeviceToHost));
    out->sweptTotal = static_cast<int64_t>(total);
    // the two smallest (error, featureIdx) keys among the exactly replayed candidates
    out->bestFeature = out->runnerUpFeature = -1;
    out->bestErr = out->runnerUpErr = INFINITY;
    const int nc = static_cast<int>(std::min<int64_t>(p.ncand, t->scratchFeat));
    if (nc > 0) {
        std::vector<unsigned long long> keys(static_cast<size_t>(nc));
        VJ_CUDA_TRY(cudaMemcpy(keys.data(), t->d_candKey, sizeof(unsigned long long) * keys.size(),
                               cudaMemcpyDeviceToHost));
        std::partial_sort(keys.begin(), keys.begin() + std::min(nc, 2), keys.end());
        for (int k = 0; k < std::min(nc, 2); ++k) {
            if (keys[static_cast<size_t>(k)] == ~0ull) break;
            const float e = bits_float(static_cast<int32_t>(keys[static_cast<size_t>(k)] >> 32));
            const int f = static_cast<int>(keys[static_cast<size_t>(k)] & 0xFFFFFFFFull) + static_cast<int>(range_begin(t));
            if (k == 0) {
                out->bestErr = e;
                out->bestFeature = f;
            } else {
                out->runnerUpErr = e;
                out->runnerUpFeature = f;
            }
        }
    }
    return ok();
}

int vj_trainer_stage_bytes(vj_trainer* t, int n, int64_t* bytes) {
    if (!t || !bytes || n <= 0) return set_error(VJ_INVALID_ARG, "vj_trainer_stage_bytes: bad arguments");
    *bytes = range_count(t) * (static_cast<int64_t>(lane_run(n)) * (32 * 2 + 2 * 2));
    return ok();
}

int vj_trainer_prepare_stage(vj_trainer* t, void* stream) {
    int st = check_bound(t, "vj_trainer_prepare_stage");
    if (st != VJ_OK) return st;
    st = sort_all(t, static_cast<cudaStream_t>(stream));
    if (st != VJ_OK) return st;
    t->prepared = true;
    t->pruneReset = true;
    return ok();
}

int vj_trainer_set_search_range(vj_trainer* t, int64_t featureBegin, int64_t featureCount) {
    if (!t || !t->d_feat) return set_error(VJ_INVALID_ARG, "vj_trainer_set_search_range: no feature pool set");
    if (featureBegin < 0 || featureCount <= 0 || featureBegin + featureCount > t->nFeat)
        return set_error(VJ_INVALID_ARG, "vj_trainer_set_search_range: range outside the feature pool");
    t->rangeBegin = featureBegin;
    t->rangeCount = featureCount;
    t->prepared = false;
    t->pruneReset = true;
    return ok();
}

int vj_reduce_tile_best(const vj_tile_best* d_in, int count, vj_tile_best* d_out, void* stream) {
    if (!d_in || !d_out || count <= 0) return set_error(VJ_INVALID_ARG, "vj_reduce_tile_best: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("reduce_tile_best_kernel", s, reduce_tile_best_kernel<<<1, 32, 0, s>>>(d_in, count, d_out));
    VJ_LAUNCH_CHECK("reduce_tile_best_kernel");
    return ok();
}

int vj_trainer_set_stage_gate(vj_trainer* t, int* d_gate) {
    if (!t) return set_error(VJ_INVALID_ARG, "vj_trainer_set_stage_gate: null trainer");
    t->d_gate = d_gate;
    return ok();
}

int vj_stump_search(vj_trainer* t, const uint8_t* d_usedMask, vj_tile_best* d_out, void* stream) {
    int st = check_bound(t, "vj_stump_search");
    if (st != VJ_OK) return st;
    if (!d_out) return set_error(VJ_INVALID_ARG, "vj_stump_search: null output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!t->prepared) {
        st = sort_all(t, s);
        if (st != VJ_OK) return st;
    }
    st = ensure_round_scratch(t);
    if (st != VJ_OK) return st;
    const int F = static_cast<int>(range_count(t)), n = t->n;
    const int fb = static_cast<int>(range_begin(t));
    const uint8_t* usedRange = d_usedMask ? d_usedMask + fb : nullptr;
    if (t->pruneReset) {
        VJ_CUDA_TRY(cudaMemsetAsync(t->d_prune, 0, sizeof(PruneState), s));
        t->pruneReset = false;
    }
    VJ_TIMED_LAUNCH("prep_round_kernel", s,
                    prep_round_kernel<<<(n + 1023) / 1024, 1024, 0, s>>>(
                        t->d_label, t->d_active, t->d_weight, n, t->d_wsg, t->d_prm, t->d_wShadow, t->d_aShadow,
                        t->d_prune, t->d_gate, t->d_prepPart, t->d_prepDone));
    VJ_LAUNCH_CHECK("prep_round_kernel");
    const bool smemW = n <= kSmemWeightsMax;
    const int sb = t->slotBase;
    // one copy of the weights per 512-thread block (two blocks per SM), or
    // both copies in one 1024-thread block per SM
    const size_t wbytes = !smemW ? 0 : sizeof(float) * (static_cast<size_t>(zero_slot(n, sb)) + 1);
    {
        const int tpb = sb > 0 ? 1024 : kSweepThreads;
        const int grid = std::min(div_up(F, tpb / 32), (1024 / tpb) * sm_count());
        auto k = sb > 0 ? sweep_kernel<true, 1024>
                        : (smemW ? sweep_kernel<true, kSweepThreads> : sweep_kernel<false, kSweepThreads>);
        VJ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(wbytes)));
        VJ_TIMED_LAUNCH("sweep_kernel", s,
                        k<<<grid, tpb, wbytes, s>>>(t->d_ord, t->ordStride, t->d_gap, t->gapStride, t->d_wsg, n, sb,
                                                    t->laneRun, F, usedRange, t->d_prm, t->d_fastErr, t->d_lb,
                                                    t->d_sweptTotal, t->d_gate));
        VJ_LAUNCH_CHECK("sweep_kernel");
    }
    VJ_TIMED_LAUNCH("select_candidates_kernel", s,
                    select_candidates_kernel<<<std::min(div_up(F, 256), 4 * sm_count()), 256, 0, s>>>(
                        t->d_fastErr, F, t->d_prm, t->d_cand, t->d_gate));
    VJ_LAUNCH_CHECK("select_candidates_kernel");
    if (n <= kRefineSplitMaxN) {
        auto k = sb > 0 ? refine_split_kernel<true> : refine_split_kernel<false>;
        const size_t nv = static_cast<size_t>((n + 255) / 256) * 256;
        const size_t lbytes = sizeof(float) * (2 * nv + 16) + sizeof(uint32_t) * (nv / 32);
        VJ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(lbytes)));
        VJ_TIMED_LAUNCH("refine_kernel", s,
                        k<<<refine_blocks(), kRefineThreads, lbytes, s>>>(
                            t->d_ord, t->ordStride, t->d_gap, t->gapStride, t->d_wsg, n, sb, t->laneRun, t->d_prm,
                            t->d_cand, t->d_refParity, t->d_refSplit, t->d_candKey, t->d_gate));
        VJ_LAUNCH_CHECK("refine_split_kernel");
    } else {
        auto k = smemW ? refine_kernel<true> : refine_kernel<false>;
        VJ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(wbytes)));
        VJ_TIMED_LAUNCH("refine_kernel", s,
                        k<<<refine_blocks(), kRefineThreads, wbytes, s>>>(
                            t->d_ord, t->ordStride, t->d_gap, t->gapStride, t->d_wsg, n, sb, t->laneRun, t->d_prm,
                            t->d_cand,
                            t->d_refParity, t->d_refSplit, t->d_candKey, t->d_prefix, static_cast<int64_t>(t->maxSamples),
                            t->d_gate));
        VJ_LAUNCH_CHECK("refine_kernel");
    }
    VJ_TIMED_LAUNCH("finalize_kernel", s,
                    finalize_kernel<<<1, 32, 0, s>>>(t->d_feat + fb, fb, t->d_sumT, t->d_invNorm, n, t->d_ord,
                                                     t->ordStride,
                                                     sb, t->laneRun, t->d_prm, t->d_refParity, t->d_refSplit, d_out,
                                                     t->d_gate));
    VJ_LAUNCH_CHECK("finalize_kernel");
    return ok();
}

int vj_round_update(vj_trainer* t, const vj_tile_best* d_best, float* d_strong, uint8_t* d_usedMask,
                    vj_weak_classifier* d_weak_out, void* stream) {
    int st = check_bound(t, "vj_round_update");
    if (st != VJ_OK) return st;
    if (!d_best || !d_strong) return set_error(VJ_INVALID_ARG, "vj_round_update: null argument");
    st = ensure_round_scratch(t);
    if (st != VJ_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("round_update_kernel", s,
                    round_update_kernel<<<div_up(t->n, kRoundPartials), kRoundPartials, 0, s>>>(
                        t->d_feat, d_best, t->d_sumT, t->d_invNorm, t->d_label, t->d_active, t->d_weight, d_strong,
                        t->n, d_usedMask, d_weak_out, t->d_status, t->d_xbuf, t->d_partials, t->d_prune,
                        t->d_gate, t->d_updDone));
    VJ_LAUNCH_CHECK("round_update_kernel");
    VJ_TIMED_LAUNCH("round_normalize_kernel", s,
                    round_normalize_kernel<<<std::min(div_up(t->n, 256), 2 * sm_count()), 256, 0, s>>>(
                        d_best, t->d_xbuf, t->d_partials, t->d_weight, t->n, t->d_wShadow, t->d_prune,
                        t->d_gate));
    VJ_LAUNCH_CHECK("round_normalize_kernel");
    return ok();
}

int vj_stage_calibrate(vj_trainer* t, const float* d_strong, int numPos, float minHitRate, float maxFalseAlarm,
                       int stageNegBaseCount, vj_stage_calib* d_out, void* stream) {
    if (!t || !d_strong || !d_out || t->n <= 0)
        return set_error(VJ_INVALID_ARG, "vj_stage_calibrate: bad arguments");
    if (numPos <= 0 || numPos > t->n || stageNegBaseCount <= 0 || !(minHitRate > 0.0f && minHitRate <= 1.0f))
        return set_error(VJ_INVALID_ARG, "vj_stage_calibrate: bad counts or hit rate");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("stage_calib_kernel", s,
                    stage_calib_kernel<<<1, 1024, 0, s>>>(d_strong, t->d_active, t->n, numPos, minHitRate,
                                                          maxFalseAlarm, stageNegBaseCount, d_out, t->d_gate));
    VJ_LAUNCH_CHECK("stage_calib_kernel");
    return ok();
}

int vj_trainer_evaluate_responses(vj_trainer* t, int featureBegin, int featureCount, float* d_out, void* stream) {
    int st = check_bound(t, "vj_trainer_evaluate_responses");
    if (st != VJ_OK) return st;
    if (!d_out || featureBegin < 0 || featureCount <= 0 || featureBegin + static_cast<int64_t>(featureCount) > t->nFeat ||
        featureCount > 65535)
        return set_error(VJ_INVALID_ARG, "vj_trainer_evaluate_responses: bad feature range");
    const dim3 grid(div_up(t->n, 256), featureCount);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("eval_responses_kernel", s,
                    eval_responses_kernel<<<grid, 256, 0, s>>>(t->d_feat, featureBegin, featureCount, t->d_sumT,
                                                               t->d_invNorm, t->n, d_out));
    VJ_LAUNCH_CHECK("eval_responses_kernel");
    return ok();
}

int vj_trainer_sort_per_feature(vj_trainer* t, const float* d_resp, int featureCount, uint16_t* d_sortedIdx,
                                void* stream) {
    if (!t || !d_resp || !d_sortedIdx || featureCount <= 0 || t->n <= 0)
        return set_error(VJ_INVALID_ARG, "vj_trainer_sort_per_feature: bad arguments");
    int st = ensure_sort_scratch(t, t->n);
    if (st != VJ_OK) return st;
    st = launch_eval_sort(nullptr, 0, featureCount, nullptr, nullptr, t->n, d_resp, d_sortedIdx, t->n, false, nullptr,
                          0, 0, 16, t->d_sortKeys, t->d_sortIdx, static_cast<cudaStream_t>(stream));
    return st == VJ_OK ? ok() : st;
}

int vj_trainer_find_thresholds(vj_trainer* t, const float* d_resp, const uint16_t* d_sortedIdx, int featureCount,
                               vj_feature_best_split* d_out, void* stream) {
    int st = check_bound(t, "vj_trainer_find_thresholds");
    if (st != VJ_OK) return st;
    if (!d_resp || !d_sortedIdx || !d_out || featureCount <= 0)
        return set_error(VJ_INVALID_ARG, "vj_trainer_find_thresholds: bad arguments");
    st = ensure_round_scratch(t);
    if (st != VJ_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("prep_round_kernel", s,
                    prep_round_kernel<<<(t->n + 1023) / 1024, 1024, 0, s>>>(
                        t->d_label, t->d_active, t->d_weight, t->n, t->d_wsg, t->d_prm, nullptr, nullptr, nullptr,
                        nullptr, t->d_prepPart, t->d_prepDone));
    VJ_LAUNCH_CHECK("prep_round_kernel");
    VJ_TIMED_LAUNCH("find_thresholds_kernel", s,
                    find_thresholds_kernel<<<div_up(featureCount, 8), 256, 0, s>>>(d_resp, d_sortedIdx, t->n,
                                                                                  featureCount, t->d_wsg, t->d_prm,
                                                                                  d_out));
    VJ_LAUNCH_CHECK("find_thresholds_kernel");
    return ok();
}

int vj_trainer_select_best_in_tile(vj_trainer* t, const vj_feature_best_split* d_best, int featureBegin,
                                   int featureCount, const uint8_t* d_usedMask, vj_tile_best* d_out, void* stream) {
    if (!t || !d_best || !d_out || featureBegin < 0 || featureCount <= 0)
        return set_error(VJ_INVALID_ARG, "vj_trainer_select_best_in_tile: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VJ_TIMED_LAUNCH("select_tile_kernel", s,
                    select_tile_kernel<<<1, 256, 0, s>>>(d_best, featureBegin, featureCount, d_usedMask, d_out));
    VJ_LAUNCH_CHECK("select_tile_kernel");
    return ok();
}

}  // extern "C"
