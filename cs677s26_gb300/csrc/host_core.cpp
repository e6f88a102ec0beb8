// Host-side pieces of libvjgb that are not kernels: error reporting, the Haar
// feature pool enumeration and the cascade_model.bin reader/writer.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"

namespace vjgb {

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

int ok() {
    g_last_error.clear();
    return VJ_OK;
}

// ---------------------------------------------------------------------------
// Haar pool.  The enumeration order, rectangle geometry and weights are those
// of FaceVisionEngine::buildHaarFeaturePool (src/face_vision_engine.cu:882-1020)
// because featureIdx values (and the index tie-break of the stump search) are
// part of the model-file contract.  Each template is one row of a table: its
// extent conditions and up to three rectangles, all linear in (dx, dy).
// ---------------------------------------------------------------------------
namespace {

struct RectSpec {
    // x = X + ax*dx + bx*dy, y = Y + ay*dx + by*dy,
    // w = aw*dx + bw*dy,     h = ah*dx + bh*dy
    int8_t ax, bx, ay, by, aw, bw, ah, bh;
    float weight;
};

struct TemplateSpec {
    int8_t right_dx;   // requires X + right_dx*dx <= W
    int8_t bottom_dx;  // requires Y + bottom_dx*dx + bottom_dy*dy <= H
    int8_t bottom_dy;
    int8_t left_dy;    // tilted only: requires X - left_dy*dy >= 0
    bool tilted;
    int8_t nrect;
    RectSpec r[3];
};

// Basic: x2, y2, x3 (+2 inner weight, face_vision_engine.cu:947-950), y3, checker.
const TemplateSpec kBasic[] = {
    {2, 0, 1, 0, false, 2, {{0, 0, 0, 0, 2, 0, 0, 1, -1.f}, {1, 0, 0, 0, 1, 0, 0, 1, 2.f}}},
    {1, 0, 2, 0, false, 2, {{0, 0, 0, 0, 1, 0, 0, 2, -1.f}, {0, 0, 0, 1, 1, 0, 0, 1, 2.f}}},
    {3, 0, 1, 0, false, 2, {{0, 0, 0, 0, 3, 0, 0, 1, -1.f}, {1, 0, 0, 0, 1, 0, 0, 1, 2.f}}},
    {1, 0, 3, 0, false, 2, {{0, 0, 0, 0, 1, 0, 0, 3, -1.f}, {0, 0, 0, 1, 1, 0, 0, 1, 2.f}}},
    {2, 0, 2, 0, false, 3,
     {{0, 0, 0, 0, 2, 0, 0, 2, -1.f}, {0, 0, 0, 0, 1, 0, 0, 1, 2.f}, {1, 0, 0, 1, 1, 0, 0, 1, 2.f}}},
};
// Core additions: x4, y4, centre-surround (+9).
const TemplateSpec kCore[] = {
    {4, 0, 1, 0, false, 2, {{0, 0, 0, 0, 4, 0, 0, 1, -1.f}, {1, 0, 0, 0, 2, 0, 0, 1, 2.f}}},
    {1, 0, 4, 0, false, 2, {{0, 0, 0, 0, 1, 0, 0, 4, -1.f}, {0, 0, 0, 1, 1, 0, 0, 2, 2.f}}},
    {3, 0, 3, 0, false, 2, {{0, 0, 0, 0, 3, 0, 0, 3, -1.f}, {1, 0, 0, 1, 1, 0, 0, 1, 9.f}}},
};
// All additions: six 45-degree templates.
const TemplateSpec kTilted[] = {
    {2, 2, 1, 1, true, 2, {{0, 0, 0, 0, 2, 0, 0, 1, -1.f}, {0, 0, 0, 0, 1, 0, 0, 1, 2.f}}},
    {1, 1, 2, 2, true, 2, {{0, 0, 0, 0, 1, 0, 0, 2, -1.f}, {0, 0, 0, 0, 1, 0, 0, 1, 2.f}}},
    {3, 3, 1, 1, true, 2, {{0, 0, 0, 0, 3, 0, 0, 1, -1.f}, {1, 0, 1, 0, 1, 0, 0, 1, 3.f}}},
    {1, 1, 3, 3, true, 2, {{0, 0, 0, 0, 1, 0, 0, 3, -1.f}, {0, -1, 0, 1, 1, 0, 0, 1, 3.f}}},
    {4, 4, 1, 1, true, 2, {{0, 0, 0, 0, 4, 0, 0, 1, -1.f}, {1, 0, 1, 0, 2, 0, 0, 1, 2.f}}},
    {1, 1, 4, 4, true, 2, {{0, 0, 0, 0, 1, 0, 0, 4, -1.f}, {0, -1, 0, 1, 1, 0, 0, 2, 2.f}}},
};

// Integral-image corner indices of one rectangle.  Upright: the four corners
// of the box.  Tilted: OpenCV's 45-degree corner convention.
vj_fast_rect corners(int x, int y, int w, int h, int iiW, float weight, bool tilted) {
    vj_fast_rect fr;
    if (tilted) {
        fr.p0 = y * iiW + x;
        fr.p1 = (y + h) * iiW + (x - h);
        fr.p2 = (y + w) * iiW + (x + w);
        fr.p3 = (y + w + h) * iiW + (x + w - h);
    } else {
        fr.p0 = y * iiW + x;
        fr.p1 = y * iiW + (x + w);
        fr.p2 = (y + h) * iiW + x;
        fr.p3 = (y + h) * iiW + (x + w);
    }
    fr.w = weight;
    return fr;
}

bool emit(const TemplateSpec& t, int X, int Y, int dx, int dy, int W, int H, int iiW,
          vj_haar_feature* f) {
    if (X + t.right_dx * dx > W) return false;
    if (Y + t.bottom_dx * dx + t.bottom_dy * dy > H) return false;
    if (t.tilted && X - t.left_dy * dy < 0) return false;
    if (!f) return true;
    vj_fast_rect rr[3];
    std::memset(rr, 0, sizeof(rr));
    for (int i = 0; i < t.nrect; ++i) {
        const RectSpec& s = t.r[i];
        rr[i] = corners(X + s.ax * dx + s.bx * dy, Y + s.ay * dx + s.by * dy,
                        s.aw * dx + s.bw * dy, s.ah * dx + s.bh * dy, iiW, s.weight, t.tilted);
    }
    f->r0 = rr[0];
    f->r1 = rr[1];
    f->r2 = rr[2];
    f->rectCount = static_cast<uint8_t>(t.nrect);
    f->tilted = t.tilted ? 1 : 0;
    f->reserved = 0;
    return true;
}

}  // namespace

int64_t build_feature_pool(int mode, int W, int H, vj_haar_feature* out, int64_t cap) {
    const int iiW = W + 1;
    int64_t n = 0;
    for (int X = 0; X < W; ++X) {
        for (int Y = 0; Y < H; ++Y) {
            for (int dx = 1; dx <= W; ++dx) {
                for (int dy = 1; dy <= H; ++dy) {
                    auto take = [&](const TemplateSpec& t) {
                        vj_haar_feature* dst = (out && n < cap) ? out + n : nullptr;
                        if (emit(t, X, Y, dx, dy, W, H, iiW, dst)) ++n;
                    };
                    for (const auto& t : kBasic) take(t);
                    if (mode != VJ_FEATURES_BASIC)
                        for (const auto& t : kCore) take(t);
                    if (mode == VJ_FEATURES_ALL)
                        for (const auto& t : kTilted) take(t);
                }
            }
        }
    }
    return n;
}

}  // namespace vjgb

using namespace vjgb;

namespace {
const char kBuildInfo[] = "vjgb: sm_103a kernels, host C++17";

// Header of cascade_model.bin: 48 bytes, little-endian, natural alignment
// (src/model_io.cpp:15-28).  The 4 bytes after winH are padding written as 0.
struct FileHeader {
    char magic[8];
    uint32_t version;
    int32_t winW;
    int32_t winH;
    uint32_t pad;
    uint64_t featureCount;
    uint64_t stumpCount;
    uint64_t stageCount;
};
static_assert(sizeof(FileHeader) == 48, "model header is 48 bytes");
const char kMagic[8] = {'V', 'J', 'C', 'B', 'I', 'N', '1', '\0'};

int read_header(FILE* fp, FileHeader* h, const char* path) {
    if (std::fread(h, sizeof(*h), 1, fp) != 1)
        return set_error(VJ_INVALID_ARG, std::string("model file too short: ") + path);
    if (std::memcmp(h->magic, kMagic, 8) != 0 || h->version != 1u)
        return set_error(VJ_INVALID_ARG, std::string("not a VJCBIN1 v1 model: ") + path);
    if (h->winW <= 0 || h->winH <= 0 || h->featureCount == 0 || h->stumpCount == 0 ||
        h->stageCount == 0)
        return set_error(VJ_INVALID_ARG, std::string("model header has an empty array: ") + path);
    return VJ_OK;
}
}  // namespace

extern "C" {

const char* vj_last_error(void) { return vjgb::g_last_error.c_str(); }

const char* vj_build_info(void) { return kBuildInfo; }

int vj_feature_pool_count(int mode, int winW, int winH, int64_t* count) {
    if (!count || winW <= 0 || winH <= 0 || mode < 0 || mode > 2)
        return set_error(VJ_INVALID_ARG, "vj_feature_pool_count: bad arguments");
    *count = build_feature_pool(mode, winW, winH, nullptr, 0);
    return ok();
}

int vj_feature_pool_build(int mode, int winW, int winH, vj_haar_feature* out, int64_t capacity,
                          int64_t* count) {
    if (!count || winW <= 0 || winH <= 0 || mode < 0 || mode > 2 || capacity < 0)
        return set_error(VJ_INVALID_ARG, "vj_feature_pool_build: bad arguments");
    const int64_t n = build_feature_pool(mode, winW, winH, out, capacity);
    *count = n;
    if (out && n > capacity)
        return set_error(VJ_INVALID_ARG, "vj_feature_pool_build: capacity too small");
    return ok();
}

int vj_model_save(const char* path, int winW, int winH, const vj_haar_feature* features,
                  int64_t featureCount, const vj_stump4* stumps, int64_t stumpCount,
                  const vj_cascade_stage* stages, int64_t stageCount) {
    if (!path || !path[0] || winW <= 0 || winH <= 0 || !features || !stumps || !stages ||
        featureCount <= 0 || stumpCount <= 0 || stageCount <= 0)
        return set_error(VJ_INVALID_ARG, "vj_model_save: bad arguments");
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return set_error(VJ_RUNTIME_ERROR, std::string("cannot open for writing: ") + path);
    FileHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = 1;
    h.winW = winW;
    h.winH = winH;
    h.featureCount = static_cast<uint64_t>(featureCount);
    h.stumpCount = static_cast<uint64_t>(stumpCount);
    h.stageCount = static_cast<uint64_t>(stageCount);
    bool good = std::fwrite(&h, sizeof(h), 1, fp) == 1;
    good = good && std::fwrite(features, sizeof(vj_haar_feature), featureCount, fp) ==
                       static_cast<size_t>(featureCount);
    good = good && std::fwrite(stumps, sizeof(vj_stump4), stumpCount, fp) ==
                       static_cast<size_t>(stumpCount);
    good = good && std::fwrite(stages, sizeof(vj_cascade_stage), stageCount, fp) ==
                       static_cast<size_t>(stageCount);
    good = (std::fclose(fp) == 0) && good;
    if (!good) return set_error(VJ_RUNTIME_ERROR, std::string("short write: ") + path);
    return ok();
}

int vj_model_load_header(const char* path, int* winW, int* winH, int64_t* featureCount,
                         int64_t* stumpCount, int64_t* stageCount) {
    if (!path || !path[0]) return set_error(VJ_INVALID_ARG, "vj_model_load_header: empty path");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return set_error(VJ_INVALID_ARG, std::string("cannot open model: ") + path);
    FileHeader h;
    const int st = read_header(fp, &h, path);
    std::fclose(fp);
    if (st != VJ_OK) return st;
    if (winW) *winW = h.winW;
    if (winH) *winH = h.winH;
    if (featureCount) *featureCount = static_cast<int64_t>(h.featureCount);
    if (stumpCount) *stumpCount = static_cast<int64_t>(h.stumpCount);
    if (stageCount) *stageCount = static_cast<int64_t>(h.stageCount);
    return ok();
}

int vj_model_load(const char* path, vj_haar_feature* features, int64_t featureCap,
                  vj_stump4* stumps, int64_t stumpCap, vj_cascade_stage* stages,
                  int64_t stageCap) {
    if (!path || !path[0] || !features || !stumps || !stages)
        return set_error(VJ_INVALID_ARG, "vj_model_load: bad arguments");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return set_error(VJ_INVALID_ARG, std::string("cannot open model: ") + path);
    FileHeader h;
    int st = read_header(fp, &h, path);
    if (st == VJ_OK && (h.featureCount > static_cast<uint64_t>(featureCap) ||
                        h.stumpCount > static_cast<uint64_t>(stumpCap) ||
                        h.stageCount > static_cast<uint64_t>(stageCap)))
        st = set_error(VJ_INVALID_ARG, "vj_model_load: output arrays smaller than the model");
    if (st == VJ_OK) {
        const bool good =
            std::fread(features, sizeof(vj_haar_feature), h.featureCount, fp) == h.featureCount &&
            std::fread(stumps, sizeof(vj_stump4), h.stumpCount, fp) == h.stumpCount &&
            std::fread(stages, sizeof(vj_cascade_stage), h.stageCount, fp) == h.stageCount;
        if (!good) st = set_error(VJ_INVALID_ARG, std::string("truncated model file: ") + path);
    }
    std::fclose(fp);
    return st == VJ_OK ? ok() : st;
}

}  // extern "C"
