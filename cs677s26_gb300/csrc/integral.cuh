// Integral-image passes shared by vj_integral_image and the detection pyramid.
#pragma once

#include <cstdint>

#include "device_util.cuh"

namespace vjgb {

// One integral image of a w x h level, row-major (h+1) x (w+1) with row pitch
// `pitch` elements (a multiple of 4, so rows start on 16-byte boundaries).
struct IIJob {
    const uint8_t* pix;  // w x h pixels, row stride `stride`
    int64_t stride;
    uint32_t* sum;       // sums; the int32 bits of the reference's sums
    uint64_t* sq;        // exact squared sums
    int w, h;
    int64_t pitch;
    int64_t rowBase;     // first row item of this job in the row pass
    int64_t itemBase;    // first work item of this job in the column passes
    int64_t totBase;     // first segment-total row of this job
};

constexpr int kColSeg = 32;  // rows per segment of the column passes

inline int64_t ii_pitch(int w) { return (static_cast<int64_t>(w) + 1 + 3) & ~int64_t(3); }
inline int col_chunks(int w) { return (w + 1 + 31) / 32; }
inline int col_segs(int h) { return (h + kColSeg - 1) / kColSeg; }

struct IIPlan {
    int64_t rows;      // row-pass items
    int64_t items;     // column-pass items (one warp each)
    int64_t totRows;   // segment-total rows
    int64_t totPitch;  // columns per segment-total row
};

// Fills the bases of each job and returns the sizes of the passes.
IIPlan plan_integral_jobs(IIJob* jobs, int njobs);

// Row pass (zero row + exclusive row prefixes) and the two column passes over
// `njobs` device-resident jobs.  d_totS / d_totQ hold totRows * totPitch
// entries.
int launch_integral_jobs(const IIJob* d_jobs, int njobs, const IIPlan& plan, uint32_t* d_totS,
                         uint64_t* d_totQ, cudaStream_t stream);

}  // namespace vjgb
