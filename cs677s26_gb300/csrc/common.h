// Internal helpers shared by the host and device translation units of libvjgb.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/vjgb.h"

namespace vjgb {

static_assert(sizeof(vj_fast_rect) == 20, "FastRect layout");
static_assert(sizeof(vj_haar_feature) == 64, "HaarFeature layout");
static_assert(sizeof(vj_stump4) == 16 && alignof(vj_stump4) == 16, "GpuStump4 layout");
static_assert(sizeof(vj_cascade_stage) == 12, "CascadeStage layout");
static_assert(sizeof(vj_detection) == 24, "Detection layout");
static_assert(sizeof(vj_tile_best) == 16, "TileBestCandidate layout");
static_assert(sizeof(vj_feature_best_split) == 16, "FeatureBestSplit layout");
static_assert(sizeof(vj_weak_classifier) == 28, "WeakClassifier layout");
static_assert(sizeof(vj_detect_stats) == 160 && sizeof(vj_detect_config) == 24, "detection record layouts");
static_assert(sizeof(vj_round_info) == 56, "round statistics layout");
static_assert(sizeof(vj_server_config) == 72 && sizeof(vj_server_stats) == 112, "server record layouts");

// Records a message for vj_last_error() and returns `status`.
int set_error(int status, const std::string& msg);
// Clears the per-thread message and returns VJ_OK.
int ok();

// Training patches are 24x24 windows; their integral image is 25x25.
constexpr int kWin = 24;
constexpr int kIIW = kWin + 1;
constexpr int kIIArea = kIIW * kIIW;  // 625
constexpr int kMaxSamples = 65535;    // 16-bit sample indices (boosting_core.cu:704)

// Host enumeration of the Haar pool in the reference order (x, y, dx, dy, type).
int64_t build_feature_pool(int mode, int winW, int winH, vj_haar_feature* out, int64_t cap);

inline int32_t float_bits(float f) {
    int32_t i;
    __builtin_memcpy(&i, &f, 4);
    return i;
}
inline float bits_float(int32_t i) {
    float f;
    __builtin_memcpy(&f, &i, 4);
    return f;
}

}  // namespace vjgb
