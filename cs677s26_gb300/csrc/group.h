// Host post-processing of raw detections.
#pragma once

#include <vector>

#include "common.h"

namespace vjgb {

// Sorts raw detections into the reference CPU path's scan order (pyramid
// level, then y, then x; main.cu:765-818).  Stable LSD radix sort.
void canonical_sort(std::vector<vj_detection>& v);

// groupRectangles (face_vision_engine.cu:1401-1539).  With threads > 1 the
// search for similar pairs of a large list is split over threads; the unions
// are still applied in the reference's sweep order.
std::vector<vj_detection> group_rectangles(const std::vector<vj_detection>& in, int minNeighbors, float eps,
                                           int threads = 1);

}  // namespace vjgb
