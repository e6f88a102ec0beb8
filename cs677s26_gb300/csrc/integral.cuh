// Integral-image passes shared by vj_integral_image and the detection pyramid.
#pragma once

#include <cstdint>

#include "device_util.cuh"

namespace vjgb {

// One integral image of a w x h level, row-major (h+1) x (w+1) with row pitch
// `pitch` elements (a multiple of 4, so rows start on 16-byte boundaries).
// Q is the element type of the squared sums: uint64_t for the exact sums of
// vj_integral_image; uint32_t (the sums modulo 2^32) for the detection
// levels, whose only use of them is the variance gate's sum over the inner
// (winW - 2) x (winH - 2) pixels of a window: below 62^2 * 255^2 < 2^32 for
// the largest window a detector accepts (64 x 64), so the four-corner
// difference modulo 2^32 is exact.
template <class Q>
struct IIJobT {
    const uint8_t* pix;  // w x h pixels, row stride `stride`
    int64_t stride;
    uint32_t* sum;       // sums; the int32 bits of the reference's sums
    Q* sq;               // squared sums
    int w, h;
    int64_t pitch;
    int64_t rowBase;     // first row item of this job in the row pass
    int64_t itemBase;    // first work item of this job in the column passes
    int64_t totBase;     // first segment-total row of this job
    int64_t walkBase;    // first item of this job in the column walk (one per 32-column chunk)
};
using IIJob = IIJobT<uint64_t>;
using IIJob32 = IIJobT<uint32_t>;

constexpr int kColSeg = 32;  // rows per segment of the column passes

inline int64_t ii_pitch(int w) { return (static_cast<int64_t>(w) + 1 + 3) & ~int64_t(3); }
inline int col_chunks(int w) { return (w + 1 + 31) / 32; }
inline int col_segs(int h) { return (h + kColSeg - 1) / kColSeg; }

struct IIPlan {
    int64_t rows;       // row-pass items
    int64_t items;      // column-pass items (one warp each)
    int64_t totRows;    // segment-total rows
    int64_t totPitch;   // columns per segment-total row
    int64_t walkItems;  // column-walk items (one warp per 32-column chunk)
};

// Fills the bases of each job and returns the sizes of the passes.
template <class Q>
IIPlan plan_integral_jobs(IIJobT<Q>* jobs, int njobs) {
    IIPlan p{0, 0, 0, 0, 0};
    for (int i = 0; i < njobs; ++i) {
        IIJobT<Q>& J = jobs[i];
        J.rowBase = p.rows;
        J.itemBase = p.items;
        J.totBase = p.totRows;
        J.walkBase = p.walkItems;
        p.walkItems += col_chunks(J.w);
        p.rows += J.h + 1;
        p.items += static_cast<int64_t>(col_chunks(J.w)) * col_segs(J.h);
        p.totRows += col_segs(J.h);
        const int64_t cols = static_cast<int64_t>(col_chunks(J.w)) * 32;
        if (cols > p.totPitch) p.totPitch = cols;
    }
    return p;
}

// Row pass (zero row + exclusive row prefixes) and the two column passes over
// `njobs` device-resident jobs.  d_totS / d_totQ hold totRows * totPitch
// entries.
int launch_integral_jobs(const IIJob* d_jobs, int njobs, const IIPlan& plan, uint32_t* d_totS,
                         uint64_t* d_totQ, cudaStream_t stream);

}  // namespace vjgb
