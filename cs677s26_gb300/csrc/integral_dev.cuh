// Device bodies of the detection-level integral passes, one work item per
// warp.  The standalone kernels of integral.cu and the persistent detection
// kernel of detect.cu call the same functions, so a level's integral image is
// computed by one piece of code whichever path runs it.
//
// Loads of pixels and integral rows are plain (coherent) global loads: in the
// persistent kernel they read data written earlier in the same launch.
#pragma once

#include "integral.cuh"

namespace vjgb {

// The job of a work item: by row-pass row (`base` 0), column-pass item (1) or
// column-walk item (2).
template <class Q>
__device__ __forceinline__ int ii_find_job(const IIJobT<Q>* __restrict__ jobs, int njobs, int64_t item, int base) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int64_t b = base == 0 ? jobs[mid].rowBase : (base == 1 ? jobs[mid].itemBase : jobs[mid].walkBase);
        if (b <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Row pass item r: integral row 0 is zero; row y >= 1 holds, at column c, the
// sum of pixels [0, c) of image row y-1 (and the sum of their squares).
// 16 pixels per lane, warp shuffle scan, 16-byte stores where aligned.
template <class Q>
__device__ __forceinline__ void ii_row_item(const IIJobT<Q>* __restrict__ jobs, int njobs, int64_t r, int lane) {
    const IIJobT<Q> J = jobs[ii_find_job(jobs, njobs, r, 0)];
    const int y = static_cast<int>(r - J.rowBase);
    uint32_t* srow = J.sum + static_cast<size_t>(y) * J.pitch;
    Q* qrow = J.sq + static_cast<size_t>(y) * J.pitch;
    const bool vecOut = ((J.pitch & 3) == 0) && ((reinterpret_cast<uintptr_t>(J.sum) & 15) == 0) &&
                        ((reinterpret_cast<uintptr_t>(J.sq) & 15) == 0);
    const uint8_t* prow = y > 0 ? J.pix + static_cast<size_t>(y - 1) * J.stride : nullptr;
    uint32_t carryS = 0, carryQ = 0;
    for (int cb = 0; cb <= J.w; cb += 512) {
        const int c0 = cb + lane * 16;
        uint32_t p[16];
        if (y == 0) {
#pragma unroll
            for (int i = 0; i < 16; ++i) p[i] = 0;
        } else if (c0 + 16 <= J.w && ((reinterpret_cast<uintptr_t>(prow + c0) & 15) == 0)) {
            const uint4 v = *reinterpret_cast<const uint4*>(prow + c0);
            const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 16; ++i) p[i] = (wv[i >> 2] >> (8 * (i & 3))) & 0xFFu;
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) p[i] = (c0 + i < J.w) ? prow[c0 + i] : 0u;
        }
        uint32_t es[16], eq[16];
        uint32_t ls = 0, lq = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            es[i] = ls;
            eq[i] = lq;
            ls += p[i];
            lq += p[i] * p[i];
        }
        uint32_t is = ls, iq = lq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ys = __shfl_up_sync(0xffffffffu, is, o);
            const uint32_t yq = __shfl_up_sync(0xffffffffu, iq, o);
            if (lane >= o) {
                is += ys;
                iq += yq;
            }
        }
        const uint32_t bs = carryS + is - ls, bq = carryQ + iq - lq;
        carryS += __shfl_sync(0xffffffffu, is, 31);
        carryQ += __shfl_sync(0xffffffffu, iq, 31);
        if (vecOut && c0 + 15 <= J.w) {
            uint4* so = reinterpret_cast<uint4*>(srow + c0);
#pragma unroll
            for (int i = 0; i < 4; ++i)
                so[i] = make_uint4(bs + es[4 * i], bs + es[4 * i + 1], bs + es[4 * i + 2], bs + es[4 * i + 3]);
            if constexpr (sizeof(Q) == 8) {
                ulonglong2* qo = reinterpret_cast<ulonglong2*>(qrow + c0);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    qo[i] = make_ulonglong2(static_cast<uint64_t>(bq + eq[2 * i]),
                                            static_cast<uint64_t>(bq + eq[2 * i + 1]));
            } else {
                uint4* qo = reinterpret_cast<uint4*>(qrow + c0);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    qo[i] = make_uint4(bq + eq[4 * i], bq + eq[4 * i + 1], bq + eq[4 * i + 2], bq + eq[4 * i + 3]);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                if (c0 + i <= J.w) {
                    srow[c0 + i] = bs + es[i];
                    qrow[c0 + i] = static_cast<Q>(bq + eq[i]);
                }
            }
        }
    }
}

template <class Q>
__device__ __forceinline__ void ii_col_item(const IIJobT<Q>& J, int64_t local, int lane, int* seg, int* c, int* r0,
                                            int* r1) {
    const int chunks = (J.w + 1 + 31) >> 5;
    *seg = static_cast<int>(local / chunks);
    *c = static_cast<int>(local % chunks) * 32 + lane;
    *r0 = 1 + *seg * kColSeg;
    *r1 = min(J.h, (*seg + 1) * kColSeg);
}

// Column pass A item: per 32-row segment and column, the sum of the row
// prefixes.
template <class Q>
__device__ __forceinline__ void ii_col_total_item(const IIJobT<Q>* __restrict__ jobs, int njobs, int64_t it, int lane,
                                                  int64_t totPitch, uint32_t* __restrict__ totS,
                                                  Q* __restrict__ totQ) {
    const IIJobT<Q> J = jobs[ii_find_job(jobs, njobs, it, 1)];
    int seg, c, r0, r1;
    ii_col_item(J, it - J.itemBase, lane, &seg, &c, &r0, &r1);
    if (c > J.w) return;
    uint32_t s = 0;
    Q q = 0;
    for (int r = r0; r <= r1; ++r) {
        s += J.sum[static_cast<size_t>(r) * J.pitch + c];
        q += J.sq[static_cast<size_t>(r) * J.pitch + c];
    }
    const size_t o = static_cast<size_t>(J.totBase + seg) * totPitch + c;
    totS[o] = s;
    totQ[o] = q;
}

// Column pass B item: carry of the segments above, then the running column
// sum written in place.
template <class Q>
__device__ __forceinline__ void ii_col_scan_item(const IIJobT<Q>* __restrict__ jobs, int njobs, int64_t it, int lane,
                                                 int64_t totPitch, const uint32_t* __restrict__ totS,
                                                 const Q* __restrict__ totQ) {
    const IIJobT<Q> J = jobs[ii_find_job(jobs, njobs, it, 1)];
    int seg, c, r0, r1;
    ii_col_item(J, it - J.itemBase, lane, &seg, &c, &r0, &r1);
    if (c > J.w) return;
    uint32_t s = 0;
    Q q = 0;
    for (int k = 0; k < seg; ++k) {
        const size_t o = static_cast<size_t>(J.totBase + k) * totPitch + c;
        s += totS[o];
        q += totQ[o];
    }
    for (int r = r0; r <= r1; ++r) {
        const size_t o = static_cast<size_t>(r) * J.pitch + c;
        s += J.sum[o];
        q += J.sq[o];
        J.sum[o] = s;
        J.sq[o] = q;
    }
}

// Column walk item (the detection levels' single column pass): one warp per
// 32-column chunk of a level, lane c down rows 1..h, adding each row prefix to
// its running column sums and writing them in place; 8 rows' loads in
// flight.  The additions are modulo 2^32 (or 2^64), so the sums equal the
// segment passes' whatever the order.
template <class Q>
__device__ __forceinline__ void ii_col_walk_item(const IIJobT<Q>* __restrict__ jobs, int njobs, int64_t it,
                                                 int lane) {
    const IIJobT<Q> J = jobs[ii_find_job(jobs, njobs, it, 2)];
    const int c = static_cast<int>(it - J.walkBase) * 32 + lane;
    if (c > J.w) return;
    const int64_t P = J.pitch;
    uint32_t* ps = J.sum + P + c;
    Q* pq = J.sq + P + c;
    uint32_t s = 0;
    Q q = 0;
    int r = 1;
    for (; r + 8 <= J.h + 1; r += 8, ps += 8 * P, pq += 8 * P) {
        uint32_t a[8];
        Q b[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            a[k] = ps[k * P];
            b[k] = pq[k * P];
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            s += a[k];
            q += b[k];
            ps[k * P] = s;
            pq[k * P] = q;
        }
    }
    for (; r <= J.h; ++r, ps += P, pq += P) {
        s += *ps;
        q += *pq;
        *ps = s;
        *pq = q;
    }
}

}  // namespace vjgb
