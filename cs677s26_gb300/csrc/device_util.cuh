// Device helpers shared by the kernels of libvjgb.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "common.h"
#include "profiler.h"

namespace vjgb {

#define VJ_CUDA_TRY(expr)                                                              \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return ::vjgb::set_error(e_ == cudaErrorMemoryAllocation ? VJ_OUT_OF_MEMORY \
                                                                     : VJ_CUDA_ERROR,  \
                                     std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define VJ_LAUNCH_CHECK(what)                                                         \
    do {                                                                              \
        cudaError_t e_ = cudaGetLastError();                                          \
        if (e_ != cudaSuccess)                                                        \
            return ::vjgb::set_error(VJ_CUDA_ERROR,                                   \
                                     std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Radix key of a float: unsigned order equals float order, -0.0 before +0.0
// (the order of a float radix sort).
__device__ __forceinline__ uint32_t radix_key(uint32_t bits) {
    return bits ^ (static_cast<uint32_t>(static_cast<int32_t>(bits) >> 31) | 0x80000000u);
}

// Inverse of radix_key: the float bits back from the order-preserving key.
__device__ __forceinline__ uint32_t radix_key_inv(uint32_t key) {
    return key ^ (static_cast<uint32_t>(static_cast<int32_t>(key ^ 0x80000000u) >> 31) | 0x80000000u);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Integral-image corner as the reference reads it: the int32 value converted
// to float with round-to-nearest (face_vision_engine.cu:474, main.cu:485-487).
__device__ __forceinline__ float corner_f(uint32_t v) { return __int2float_rn(static_cast<int32_t>(v)); }

// Training response of one feature on sample s from the transposed sums
// [625][n]: per rectangle (c0 - c1 - c2 + c3) in float, left to right, then
// w0*s0 + w1*s1 (+ w2*s2), times invNorm, each operation rounded on its own
// (main.cu:476-496, boosting_core.cu:249-260).
__device__ __forceinline__ float train_response(const vj_haar_feature& f, const uint32_t* __restrict__ sumT,
                                                int n, int s, float invNorm) {
    const size_t N = static_cast<size_t>(n);
    auto rs = [&](const vj_fast_rect& r) {
        const float a = corner_f(__ldg(sumT + static_cast<size_t>(r.p0) * N + s));
        const float b = corner_f(__ldg(sumT + static_cast<size_t>(r.p1) * N + s));
        const float c = corner_f(__ldg(sumT + static_cast<size_t>(r.p2) * N + s));
        const float d = corner_f(__ldg(sumT + static_cast<size_t>(r.p3) * N + s));
        return __fadd_rn(__fsub_rn(__fsub_rn(a, b), c), d);
    };
    const float s0 = rs(f.r0);
    const float s1 = rs(f.r1);
    float resp = __fadd_rn(__fmul_rn(f.r0.w, s0), __fmul_rn(f.r1.w, s1));
    if (f.rectCount == 3) resp = __fadd_rn(resp, __fmul_rn(f.r2.w, rs(f.r2)));
    return __fmul_rn(resp, invNorm);
}

// Corners that a feature's rectangles share, for the response evaluation:
// the same train_response arithmetic with each shared corner loaded once.
//   1: two rectangles, r1.p1 = r0.p1 and r1.p3 = r0.p3;
//   2: two rectangles, r1.p2 = r0.p2 and r1.p3 = r0.p3;
//   3: three rectangles, r1.p0 = r0.p0, r2.p0 = r1.p3 and r2.p3 = r0.p3;
//   0: anything else (every corner loaded).
// The three shapes cover every non-tilted Basic, Core and All feature that
// shares a corner.
__host__ __device__ __forceinline__ int corner_sharing(const vj_haar_feature& f) {
    if (f.rectCount == 2) {
        if (f.r1.p1 == f.r0.p1 && f.r1.p3 == f.r0.p3) return 1;
        if (f.r1.p2 == f.r0.p2 && f.r1.p3 == f.r0.p3) return 2;
    } else if (f.rectCount == 3) {
        if (f.r1.p0 == f.r0.p0 && f.r2.p0 == f.r1.p3 && f.r2.p3 == f.r0.p3) return 3;
    }
    return 0;
}

// train_response for a feature of corner_sharing(f) == S.
template <int S>
__device__ __forceinline__ float train_response_shared(const vj_haar_feature& f, const uint32_t* __restrict__ sumT,
                                                       int n, int s, float invNorm) {
    if (S == 0) return train_response(f, sumT, n, s, invNorm);
    const size_t N = static_cast<size_t>(n);
    auto ld = [&](int p) { return corner_f(__ldg(sumT + static_cast<size_t>(p) * N + s)); };
    auto rect = [](float a, float b, float c, float d) { return __fadd_rn(__fsub_rn(__fsub_rn(a, b), c), d); };
    const float a0 = ld(f.r0.p0), a1 = ld(f.r0.p1), a2 = ld(f.r0.p2), a3 = ld(f.r0.p3);
    float resp;
    if (S == 1) {
        const float b0 = ld(f.r1.p0), b2 = ld(f.r1.p2);
        resp = __fadd_rn(__fmul_rn(f.r0.w, rect(a0, a1, a2, a3)), __fmul_rn(f.r1.w, rect(b0, a1, b2, a3)));
    } else if (S == 2) {
        const float b0 = ld(f.r1.p0), b1 = ld(f.r1.p1);
        resp = __fadd_rn(__fmul_rn(f.r0.w, rect(a0, a1, a2, a3)), __fmul_rn(f.r1.w, rect(b0, b1, a2, a3)));
    } else {
        const float b1 = ld(f.r1.p1), b2 = ld(f.r1.p2), b3 = ld(f.r1.p3);
        const float c1 = ld(f.r2.p1), c2 = ld(f.r2.p2);
        resp = __fadd_rn(__fmul_rn(f.r0.w, rect(a0, a1, a2, a3)), __fmul_rn(f.r1.w, rect(a0, b1, b2, b3)));
        resp = __fadd_rn(resp, __fmul_rn(f.r2.w, rect(b3, c1, c2, a3)));
    }
    return __fmul_rn(resp, invNorm);
}

// train_response of the two consecutive samples s, s+1 (s even, sumT and
// invNorm 8-byte aligned, n even), each corner of corner_sharing shape S read
// once as one 8-byte load for both samples; every sample's arithmetic is
// train_response's.
template <int S>
__device__ __forceinline__ float2 train_response2(const vj_haar_feature& f, const uint32_t* __restrict__ sumT, int n,
                                                  int s, float2 inv) {
    static_assert(S >= 1 && S <= 3, "a sharing shape; the generic form reads every corner one sample at a time");
    const size_t N = static_cast<size_t>(n);
    auto ld = [&](int p) { return __ldg(reinterpret_cast<const uint2*>(sumT + static_cast<size_t>(p) * N + s)); };
    // the corners in train_response's order (r0.p0..p3, r1.p0..p3, r2.p0..p3)
    uint2 c[12];
    c[0] = ld(f.r0.p0);
    c[1] = ld(f.r0.p1);
    c[2] = ld(f.r0.p2);
    c[3] = ld(f.r0.p3);
    c[4] = S == 3 ? c[0] : ld(f.r1.p0);
    c[5] = S == 1 ? c[1] : ld(f.r1.p1);
    c[6] = S == 2 ? c[2] : ld(f.r1.p2);
    c[7] = (S == 1 || S == 2) ? c[3] : ld(f.r1.p3);
    constexpr bool three = S == 3;
    if (three) {
        c[8] = c[7];
        c[9] = ld(f.r2.p1);
        c[10] = ld(f.r2.p2);
        c[11] = c[3];
    }
    auto one = [&](int j, float iv) {
        auto cf = [&](int q) { return corner_f(j == 0 ? c[q].x : c[q].y); };
        auto rect = [&](int q) { return __fadd_rn(__fsub_rn(__fsub_rn(cf(q), cf(q + 1)), cf(q + 2)), cf(q + 3)); };
        float resp = __fadd_rn(__fmul_rn(f.r0.w, rect(0)), __fmul_rn(f.r1.w, rect(4)));
        if (three) resp = __fadd_rn(resp, __fmul_rn(f.r2.w, rect(8)));
        return __fmul_rn(resp, iv);
    };
    return make_float2(one(0, inv.x), one(1, inv.y));
}

inline int div_up(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace vjgb
