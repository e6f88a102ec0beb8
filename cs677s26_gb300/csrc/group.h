// Host post-processing of raw detections.
#pragma once

#include <vector>

#include "common.h"

namespace vjgb {

// Sorts raw detections into the reference CPU path's scan order (pyramid
// level, then y, then x; main.cu:765-818).  Stable LSD radix sort.
void canonical_sort(std::vector<vj_detection>& v);

// groupRectangles (face_vision_engine.cu:1401-1539).
std::vector<vj_detection> group_rectangles(const std::vector<vj_detection>& in, int minNeighbors, float eps);

}  // namespace vjgb
