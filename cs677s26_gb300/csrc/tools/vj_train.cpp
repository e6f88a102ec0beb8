// vj_train: the drop-in for `cuda_hello train` (src/main.cu:1370-2392).
//
//   vj_train [faces_u8.bin] [numNeg] [maxWeakPerStage] [maxDetections]
//            [minNeighbors] [scaleFactor] [maxStages] [minHitRate]
//            [maxFalseAlarm] [minObjectSize] [stageNegCacheDir]
//            [stageNegImagesDir] [stageNegSeed] [hardNegCandidateMultiplier]
//            <out_model.bin>
//
// Same arguments, defaults, clamps and stage loop as the reference:
//   - per stage, positives re-drawn from the pool (mt19937 shuffle, 10,000
//     at most) and 10,000 negatives: random crops at stage 0, hard negatives
//     mined with the cascade trained so far from stageNegImagesDir's PGMs
//     afterwards (top 256 windows by score per image, cropped and resized to
//     24x24), topped up with random crops;
//   - weights reset to 0.5/numPos and 0.5/numNeg, then boosting rounds over
//     the Core feature pool until the stage reaches (hit >= minHitRate and
//     false alarm <= maxFalseAlarm) or rejects every negative, at most
//     maxWeakPerStage rounds and 6,061 weak classifiers in all;
//   - the stage threshold stored is the calibrated one minus 1e-5f.
// The rounds run on the device (stage-resident sorted orders, the exact
// reference stump pick, FP64 renormalisation, on-device calibration) behind
// the trainer's stage gate, so the host reads back once per 16 queued
// rounds instead of after every round; the
// mining runs as batched detection (vj_detect_batch over 32 images per launch).
//
// Differences, all in how negatives are sourced: random crops come from this
// program's own sampler (a square of side uniform in [24, min(w, h)] at a
// uniform position, resized with the reference's crop-resize) instead of the
// reference's Python script; the PGM list is sorted before its seeded
// shuffle, so the order does not depend on the file system.  The mined
// windows are cropped on the device (vj_crop_resize_batch) from the batch's
// images, which are uploaded once for detection and cropping.  Setting
// VJ_TRAIN_DUMP=<dir> writes each stage's training patches (positives, then
// negatives) to <dir>/stageNN.bin.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "image_io.h"
#include "vjgb.h"

namespace {

using vjtools::crop_resize;
using vjtools::Gray;
using vjtools::load_pgm;

constexpr int kStages = 38;
constexpr int kTotalFeatures = 6061;
constexpr int kPosPerStage = 10000;
constexpr int kNegPerStage = 10000;
constexpr int kWin = 24;
constexpr int kPix = kWin * kWin;
constexpr int kMineBatch = 32;
constexpr int kPerImageKeep = 256;
constexpr int kMiningMax = 2048;
constexpr int kRoundChunk = 16;  // boosting rounds queued per read of the stage gate

// A raw sample file: N patches of 24x24 uint8 back to back, N from the file
// size (the reference's loadRawSampleBin, main.cu:122-162, reads the same
// format and prints the same messages).
bool load_raw_bin(const std::string& path, std::vector<uint8_t>& out, int& count) {
    switch (vjtools::read_file(path, out)) {
        case 1:
            std::cerr << "[ERR] Cannot open: " << path << "\n";
            return false;
        case 2:
            std::cerr << "[ERR] Failed to read: " << path << "\n";
            return false;
        default:
            break;
    }
    if (out.empty()) {
        std::cerr << "[ERR] Empty file: " << path << "\n";
        return false;
    }
    if (out.size() % kPix != 0) {
        std::cerr << "[ERR] File size is not divisible by samplePixels: " << path << "\n";
        return false;
    }
    count = static_cast<int>(out.size() / kPix);
    return true;
}

std::vector<std::string> collect_pgms(const std::string& root) {
    namespace fs = std::filesystem;
    std::vector<std::string> out;
    std::error_code ec;
    if (!fs::exists(root, ec)) return out;
    for (fs::recursive_directory_iterator it(root, ec), end; it != end; it.increment(ec)) {
        if (ec) break;
        if (!it->is_regular_file()) continue;
        std::string ext = it->path().extension().string();
        std::transform(ext.begin(), ext.end(), ext.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
        if (ext == ".pgm") out.push_back(it->path().string());
    }
    std::sort(out.begin(), out.end());
    return out;
}

// `count` random 24x24 negatives: images drawn uniformly, up to 50 crops per
// image visit, each a square of side uniform in [24, min(w, h)] at a uniform
// position, resized to 24x24.
bool sample_random_negatives(const std::vector<std::string>& paths, int count, uint32_t seed, std::vector<uint8_t>& out) {
    std::mt19937 rng(seed);
    std::vector<std::string> order = paths;
    std::shuffle(order.begin(), order.end(), rng);
    std::vector<Gray> usable;
    for (const auto& p : order) {
        Gray g;
        if (!load_pgm(p, g, true)) continue;
        if (std::min(g.w, g.h) < kWin) continue;
        usable.push_back(std::move(g));
        if (usable.size() >= 512) break;  // a bounded working set of decoded images
    }
    if (usable.empty()) return false;
    out.assign(static_cast<size_t>(count) * kPix, 0);
    int made = 0;
    while (made < count) {
        const Gray& g = usable[std::uniform_int_distribution<size_t>(0, usable.size() - 1)(rng)];
        const int k = std::min(count - made, 50);
        const int maxSide = std::min(g.w, g.h);
        for (int i = 0; i < k; ++i) {
            const int side = std::uniform_int_distribution<int>(kWin, maxSide)(rng);
            const int x0 = std::uniform_int_distribution<int>(0, g.w - side)(rng);
            const int y0 = std::uniform_int_distribution<int>(0, g.h - side)(rng);
            crop_resize(g, x0, y0, side, side, kWin, out.data() + static_cast<size_t>(made++) * kPix);
        }
    }
    return true;
}

template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    bool alloc(size_t count) {
        n = count;
        return cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)) == cudaSuccess;
    }
    ~DevArray() {
        if (p) cudaFree(p);
    }
};

int fail(const char* what) {
    std::cerr << "[ERR] " << what << " failed: " << vj_last_error() << "\n";
    return 1;
}

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    std::cerr << "[ERR] " << what << ": " << cudaGetErrorString(e) << "\n";
    return false;
}

}  // namespace

int main(int argc, char** argv) {
    const int modelArgIdx = argc - 1;
    if (modelArgIdx < 1) {
        std::cerr << "Usage: vj_train [faces_u8.bin] [numNeg]"
                  << " [maxWeakPerStage] [maxDetections] [minNeighbors] [scaleFactor] [maxStages]"
                  << " [minHitRate] [maxFalseAlarm] [minObjectSize]"
                  << " [stageNegCacheDir] [stageNegImagesDir] [stageNegSeed] [hardNegCandidateMultiplier]"
                  << " <out_model.bin>\n";
        return 1;
    }
    const std::string modelOutPath = argv[modelArgIdx];
    const std::string posPath = modelArgIdx > 1 ? argv[1] : "faces_u8.bin";
    int numNeg = kNegPerStage, maxWeakPerStage = 250, maxStages = kStages, maxDetections = 200000;
    int minNeighbors = 4, minObjectSize = 24, hardNegCandidateMultiplier = 3, stageNegSeed = 677;
    float scaleFactor = 1.25f, minHitRate = 0.99f, maxFalseAlarm = 0.40f;
    std::string stageNegCacheDir, stageNegImagesDir = "data_cache/coco_val2017_nonperson_pgm";
    auto argInt = [&](int i, int lo, int& dst, const char* name) {
        try {
            dst = std::max(lo, std::stoi(argv[i]));
            return true;
        } catch (...) {
            std::cerr << "[ERR] Invalid " << name << " argument: " << argv[i] << "\n";
            return false;
        }
    };
    if (modelArgIdx > 2 && !argInt(2, 1, numNeg, "numNeg")) return 1;
    if (modelArgIdx > 3 && !argInt(3, 1, maxWeakPerStage, "maxWeakPerStage")) return 1;
    if (modelArgIdx > 4 && !argInt(4, 100, maxDetections, "maxDetections")) return 1;
    if (modelArgIdx > 5 && !argInt(5, 1, minNeighbors, "minNeighbors")) return 1;
    if (modelArgIdx > 6) {
        try {
            scaleFactor = std::stof(argv[6]);
        } catch (...) {
            std::cerr << "[ERR] Invalid scaleFactor argument: " << argv[6] << "\n";
            return 1;
        }
        if (scaleFactor <= 1.0f) {
            std::cerr << "[ERR] scaleFactor must be > 1.0\n";
            return 1;
        }
    }
    if (modelArgIdx > 7 && !argInt(7, 1, maxStages, "maxStages")) return 1;
    if (modelArgIdx > 8) {
        try {
            minHitRate = std::stof(argv[8]);
        } catch (...) {
            std::cerr << "[ERR] Invalid minHitRate argument: " << argv[8] << "\n";
            return 1;
        }
        if (minHitRate <= 0.0f || minHitRate > 1.0f) {
            std::cerr << "[ERR] minHitRate must be in (0, 1]\n";
            return 1;
        }
    }
    if (modelArgIdx > 9) {
        try {
            maxFalseAlarm = std::stof(argv[9]);
        } catch (...) {
            std::cerr << "[ERR] Invalid maxFalseAlarm argument: " << argv[9] << "\n";
            return 1;
        }
        if (maxFalseAlarm < 0.0f || maxFalseAlarm > 1.0f) {
            std::cerr << "[ERR] maxFalseAlarm must be in [0, 1]\n";
            return 1;
        }
    }
    if (modelArgIdx > 10 && !argInt(10, 1, minObjectSize, "minObjectSize")) return 1;
    if (modelArgIdx > 11) stageNegCacheDir = argv[11];
    if (modelArgIdx > 12) stageNegImagesDir = argv[12];
    if (modelArgIdx > 13) {
        try {
            stageNegSeed = std::stoi(argv[13]);
        } catch (...) {
            std::cerr << "[ERR] Invalid stageNegSeed argument: " << argv[13] << "\n";
            return 1;
        }
    }
    if (modelArgIdx > 14 && !argInt(14, 1, hardNegCandidateMultiplier, "hardNegCandidateMultiplier")) return 1;
    if (numNeg != kNegPerStage) {
        std::cout << "[INFO] numNeg is fixed to paper-style per-stage setting: " << kNegPerStage << "\n";
        numNeg = kNegPerStage;
    }
    if (maxStages > kStages) {
        std::cout << "[INFO] maxStages capped to " << kStages << "\n";
        maxStages = kStages;
    }
    std::cout << "[INFO] Config: maxWeakPerStage=" << maxWeakPerStage << " maxStages=" << maxStages
              << " scaleFactor=" << scaleFactor << " minNeighbors=" << minNeighbors
              << " minObjectSize=" << minObjectSize << " maxDetections=" << maxDetections
              << " minHitRate=" << minHitRate << " maxFalseAlarm=" << maxFalseAlarm << " numNeg=" << numNeg
              << " hardNegCandMul=" << hardNegCandidateMultiplier << "\n";
    if (stageNegCacheDir.empty()) {
        std::cerr << "[ERR] stageNegCacheDir is required. Dynamic negatives are mandatory.\n";
        std::cerr << "Usage: vj_train ... <out_model.bin>\n";
        return 1;
    }
    std::vector<uint8_t> posRaw;
    int numPosPool = 0;
    if (!load_raw_bin(posPath, posRaw, numPosPool)) return 1;
    const int numPos = std::min(numPosPool, kPosPerStage);
    const int n = numPos + numNeg;
    const std::vector<std::string> pgms = collect_pgms(stageNegImagesDir);
    if (pgms.empty()) {
        std::cerr << "[ERR] No PGM images found in " << stageNegImagesDir << "\n";
        return 1;
    }
    const char* dumpDir = std::getenv("VJ_TRAIN_DUMP");

    // Feature pool (Core, as the reference's train mode, main.cu:1631).
    int64_t nf = 0;
    if (vj_feature_pool_count(VJ_FEATURES_CORE, kWin, kWin, &nf) != VJ_OK) return fail("feature pool");
    std::vector<vj_haar_feature> feats(static_cast<size_t>(nf));
    if (vj_feature_pool_build(VJ_FEATURES_CORE, kWin, kWin, feats.data(), nf, &nf) != VJ_OK)
        return fail("feature pool");
    std::cout << "[INFO] Feature count: " << nf << "\n";
    vj_trainer* tr = nullptr;
    if (vj_trainer_create(kWin, kWin, n, &tr) != VJ_OK) return fail("trainer create");
    if (vj_trainer_set_features(tr, feats.data(), nf) != VJ_OK) return fail("uploadFeaturePool");
    vj_detector* miner = nullptr;
    if (vj_detector_create(kWin, kWin, kMiningMax, kMiningMax, std::max(20000, numNeg * 2), &miner) != VJ_OK)
        return fail("mining detector create");

    DevArray<uint8_t> dTrain, dActive, dUsed, dImg;
    DevArray<uint32_t> dSumT;
    DevArray<float> dInv, dWeight, dStrong;
    DevArray<int8_t> dLabel;
    DevArray<vj_tile_best> dBest;
    DevArray<vj_weak_classifier> dWeak;  // one record per round of a stage
    DevArray<vj_stage_calib> dCalib;
    DevArray<int> dGate;
    const int maxRounds = std::min(maxWeakPerStage, kTotalFeatures);
    if (!dTrain.alloc(static_cast<size_t>(n) * kPix) || !dActive.alloc(n) || !dUsed.alloc(static_cast<size_t>(nf)) ||
        !dSumT.alloc(static_cast<size_t>(625) * n) || !dInv.alloc(n) || !dWeight.alloc(n) || !dStrong.alloc(n) ||
        !dLabel.alloc(n) || !dBest.alloc(1) || !dWeak.alloc(static_cast<size_t>(maxRounds)) ||
        !dCalib.alloc(static_cast<size_t>(maxRounds)) || !dGate.alloc(1)) {
        std::cerr << "[ERR] device allocation failed\n";
        return 1;
    }
    std::vector<int8_t> hLabel(static_cast<size_t>(n), -1);
    std::fill(hLabel.begin(), hLabel.begin() + numPos, int8_t(1));
    if (!cuda_ok(cudaMemcpy(dLabel.p, hLabel.data(), n, cudaMemcpyHostToDevice), "labels")) return 1;

    std::vector<uint8_t> trainRaw(static_cast<size_t>(n) * kPix);
    std::vector<vj_weak_classifier> weaks;
    std::vector<vj_cascade_stage> stages;
    const auto t0 = std::chrono::high_resolution_clock::now();
    std::cout << "[TRAIN] Start cascade training: maxStages=" << maxStages << " maxWeakPerStage=" << maxWeakPerStage
              << " totalFeatureBudget=" << kTotalFeatures << "\n";
    for (int stageIdx = 0; stageIdx < maxStages; ++stageIdx) {
        if (static_cast<int>(weaks.size()) >= kTotalFeatures) {
            std::cout << "[TRAIN] Reached total feature budget " << kTotalFeatures << ", stop at stage " << stageIdx
                      << "\n";
            break;
        }
        const int perStageSeed = stageNegSeed + stageIdx * 1000003;
        // positives: the whole pool, or numPos drawn by a seeded shuffle
        if (numPosPool <= numPos) {
            std::memcpy(trainRaw.data(), posRaw.data(), static_cast<size_t>(numPos) * kPix);
        } else {
            std::vector<int> idx(static_cast<size_t>(numPosPool));
            std::iota(idx.begin(), idx.end(), 0);
            std::mt19937 rng(static_cast<uint32_t>(perStageSeed ^ 0x7f4a7c15));
            std::shuffle(idx.begin(), idx.end(), rng);
            for (int i = 0; i < numPos; ++i)
                std::memcpy(trainRaw.data() + static_cast<size_t>(i) * kPix,
                            posRaw.data() + static_cast<size_t>(idx[static_cast<size_t>(i)]) * kPix, kPix);
        }
        uint8_t* negDst = trainRaw.data() + static_cast<size_t>(numPos) * kPix;
        int hard = 0;
        if (stageIdx == 0) {
            std::vector<uint8_t> neg;
            if (!sample_random_negatives(pgms, numNeg, static_cast<uint32_t>(perStageSeed), neg)) {
                std::cerr << "[ERR] stage negative sampling failed at stage " << stageIdx << "\n";
                return 1;
            }
            std::memcpy(negDst, neg.data(), neg.size());
            hard = numNeg;
        } else {
            // hard negatives: batched detection with the cascade so far
            std::vector<vj_stump4> stumps(weaks.size());
            for (size_t i = 0; i < weaks.size(); ++i) {
                float fb;
                std::memcpy(&fb, &weaks[i].featureIdx, 4);
                stumps[i] = vj_stump4{fb, weaks[i].theta, weaks[i].leftVal, weaks[i].rightVal};
            }
            if (vj_detector_set_model(miner, feats.data(), nf, stumps.data(), static_cast<int64_t>(stumps.size()),
                                      stages.data(), static_cast<int64_t>(stages.size())) != VJ_OK)
                return fail("set mining cascade model");
            std::vector<std::string> order = pgms;
            std::mt19937 mineRng(static_cast<uint32_t>(perStageSeed));
            std::shuffle(order.begin(), order.end(), mineRng);
            const int capPer = std::max(20000, numNeg * 2);
            std::vector<vj_detection> out(static_cast<size_t>(kMineBatch) * capPer);
            // a batch's images go to the device once: detection reads them
            // there and the chosen windows are cropped there
            DevArray<uint8_t> dBatch, dPatches;
            if (!dPatches.alloc(static_cast<size_t>(kMineBatch) * kPerImageKeep * kPix))
                return fail("mining patch buffer");
            int scanned = 0;
            for (size_t pos = 0; pos < order.size() && hard < numNeg;) {
                std::vector<Gray> batch;
                while (pos < order.size() && static_cast<int>(batch.size()) < kMineBatch) {
                    Gray g;
                    const std::string& p = order[pos++];
                    if (!load_pgm(p, g, true)) continue;
                    if (g.w < kWin || g.h < kWin || g.w > kMiningMax || g.h > kMiningMax) continue;
                    batch.push_back(std::move(g));
                }
                if (batch.empty()) break;
                const int bn = static_cast<int>(batch.size());
                std::vector<const uint8_t*> ptrs(bn);
                std::vector<int> ws(bn), hs(bn), counts(bn);
                size_t bytes = 0;
                for (int i = 0; i < bn; ++i) bytes += static_cast<size_t>(batch[i].w) * batch[i].h;
                if (bytes > dBatch.n) {
                    cudaFree(dBatch.p);
                    dBatch.p = nullptr;
                    if (!dBatch.alloc(bytes)) return fail("mining image buffer");
                }
                size_t off = 0;
                for (int i = 0; i < bn; ++i) {
                    ptrs[i] = dBatch.p + off;
                    ws[i] = batch[i].w;
                    hs[i] = batch[i].h;
                    if (!cuda_ok(cudaMemcpy(dBatch.p + off, batch[i].px.data(), batch[i].px.size(),
                                            cudaMemcpyHostToDevice), "mining image"))
                        return 1;
                    off += batch[i].px.size();
                }
                if (vj_detect_batch(miner, bn, ptrs.data(), ws.data(), hs.data(), ws.data(), 1, scaleFactor, 0, kWin,
                                    capPer, 0, out.data(), capPer, counts.data(), nullptr) != VJ_OK)
                    return fail("mining detectMultiScale");
                // the top windows by score of each image, in image order, up to numNeg in all
                std::vector<vj_detection> boxes;
                std::vector<int> imageOf;
                std::vector<int> scannedAt;  // crops chosen when each image is scanned
                int chosen = hard;
                for (int i = 0; i < bn && chosen < numNeg; ++i) {
                    vj_detection* d = out.data() + static_cast<size_t>(i) * capPer;
                    const int keep = std::min(counts[i], kPerImageKeep);
                    std::partial_sort(d, d + keep, d + counts[i],
                                      [](const vj_detection& a, const vj_detection& b) { return a.score > b.score; });
                    for (int k = 0; k < keep && chosen < numNeg; ++k, ++chosen) {
                        boxes.push_back(d[k]);
                        imageOf.push_back(i);
                    }
                    scannedAt.push_back(chosen);
                }
                const int nc = static_cast<int>(boxes.size());
                if (nc > 0) {
                    if (vj_crop_resize_batch(bn, ptrs.data(), ws.data(), hs.data(), ws.data(), nc, imageOf.data(),
                                             boxes.data(), kWin, dPatches.p, nullptr) != VJ_OK)
                        return fail("mining cropResizeTo24");
                    if (!cuda_ok(cudaMemcpy(negDst + static_cast<size_t>(hard) * kPix, dPatches.p,
                                            static_cast<size_t>(nc) * kPix, cudaMemcpyDeviceToHost), "mined patches"))
                        return 1;
                }
                for (const int c : scannedAt)
                    if ((++scanned % 20) == 0)
                        std::cout << "[MINE] stage=" << stageIdx << " scanned=" << scanned << " hard=" << c << "/"
                                  << numNeg << "\n";
                hard += nc;
            }
            std::cout << "[TRAIN] stage=" << stageIdx << " hardNegSelected=" << hard << "/" << numNeg << "\n";
        }
        if (hard < numNeg) {
            const int fallbackCount = std::max(numNeg, (numNeg - hard) * hardNegCandidateMultiplier);
            std::vector<uint8_t> pool;
            if (!sample_random_negatives(pgms, fallbackCount, static_cast<uint32_t>(perStageSeed ^ 0x9e3779b9), pool)) {
                std::cerr << "[ERR] fallback stage negative sampling failed at stage " << stageIdx << "\n";
                return 1;
            }
            std::mt19937 rng(static_cast<uint32_t>(perStageSeed ^ 0x5bd1e995u));
            std::uniform_int_distribution<int> pick(0, fallbackCount - 1);
            while (hard < numNeg)
                std::memcpy(negDst + static_cast<size_t>(hard++) * kPix, pool.data() + static_cast<size_t>(pick(rng)) * kPix,
                            kPix);
        }
        if (dumpDir) {
            char name[64];
            std::snprintf(name, sizeof(name), "/stage%02d.bin", stageIdx);
            std::ofstream(std::string(dumpDir) + name, std::ios::binary)
                .write(reinterpret_cast<const char*>(trainRaw.data()), static_cast<std::streamsize>(trainRaw.size()));
        }
        // stage training set on the device, weights reset and normalised
        std::vector<float> w(static_cast<size_t>(n));
        double sum = 0.0;
        for (int i = 0; i < n; ++i) {
            w[i] = i < numPos ? 0.5f / static_cast<float>(numPos) : 0.5f / static_cast<float>(numNeg);
            sum += w[i];
        }
        for (float& x : w) x = static_cast<float>(static_cast<double>(x) / sum);
        if (!cuda_ok(cudaMemcpy(dTrain.p, trainRaw.data(), trainRaw.size(), cudaMemcpyHostToDevice), "train set") ||
            !cuda_ok(cudaMemset(dActive.p, 1, n), "active") ||
            !cuda_ok(cudaMemcpy(dWeight.p, w.data(), sizeof(float) * n, cudaMemcpyHostToDevice), "weights") ||
            !cuda_ok(cudaMemset(dStrong.p, 0, sizeof(float) * n), "strong") ||
            !cuda_ok(cudaMemset(dUsed.p, 0, static_cast<size_t>(nf)), "used mask"))
            return 1;
        if (vj_integral_batch(dTrain.p, kWin, kWin, kWin, n, dSumT.p, nullptr, dInv.p, nullptr) != VJ_OK)
            return fail("computeIntegralBatchTransposed");
        if (vj_trainer_bind(tr, dSumT.p, dInv.p, n, dLabel.p, dActive.p, dWeight.p) != VJ_OK)
            return fail("bindTrainingSet");
        if (vj_trainer_prepare_stage(tr, nullptr) != VJ_OK) return fail("prepare stage");
        const int stageFirst = static_cast<int>(weaks.size());
        const int limit = std::min(maxWeakPerStage, kTotalFeatures - stageFirst);
        bool satisfied = false;
        float stageThreshold = 0.0f;
        // The rounds run behind the trainer's stage gate, queued kRoundChunk
        // at a time with one read of the gate per chunk: a round that finds
        // no valid stump or meets the stage targets closes the gate and the
        // rest of the queued rounds do nothing.  Unrun rounds keep featureIdx
        // -1 in their weak record.
        if (!cuda_ok(cudaMemset(dGate.p, 0, sizeof(int)), "gate") ||
            !cuda_ok(cudaMemset(dWeak.p, 0xFF, sizeof(vj_weak_classifier) * static_cast<size_t>(limit)), "weak records"))
            return 1;
        if (vj_trainer_set_stage_gate(tr, dGate.p) != VJ_OK) return fail("stage gate");
        int queued = 0, gate = 0;
        while (queued < limit && gate == 0) {
            const int end = std::min(limit, queued + kRoundChunk);
            for (int r = queued; r < end; ++r) {
                if (vj_stump_search(tr, dUsed.p, dBest.p, nullptr) != VJ_OK) return fail("best-weak search");
                if (vj_round_update(tr, dBest.p, dStrong.p, dUsed.p, dWeak.p + r, nullptr) != VJ_OK)
                    return fail("round update");
                if (vj_stage_calibrate(tr, dStrong.p, numPos, minHitRate, maxFalseAlarm, numNeg, dCalib.p + r,
                                       nullptr) != VJ_OK)
                    return fail("stage calibration");
            }
            queued = end;
            if (!cuda_ok(cudaMemcpy(&gate, dGate.p, sizeof(int), cudaMemcpyDeviceToHost), "gate")) return 1;
        }
        vj_trainer_set_stage_gate(tr, nullptr);
        std::vector<vj_weak_classifier> roundWeak(static_cast<size_t>(queued));
        std::vector<vj_stage_calib> roundCal(static_cast<size_t>(queued));
        if (!cuda_ok(cudaMemcpy(roundWeak.data(), dWeak.p, sizeof(vj_weak_classifier) * roundWeak.size(),
                                cudaMemcpyDeviceToHost), "weak records") ||
            !cuda_ok(cudaMemcpy(roundCal.data(), dCalib.p, sizeof(vj_stage_calib) * roundCal.size(),
                                cudaMemcpyDeviceToHost), "calibrations"))
            return 1;
        for (int r = 0; r < queued; ++r) {
            const vj_weak_classifier& wk = roundWeak[static_cast<size_t>(r)];
            const vj_stage_calib& cal = roundCal[static_cast<size_t>(r)];
            if (wk.featureIdx < 0) {
                std::cerr << "[WARN] No valid weak found at stage " << stageIdx << " weakRound " << r << "\n";
                break;
            }
            weaks.push_back(wk);
            stageThreshold = cal.stageThreshold;
            std::cout << "[TRAIN] stage=" << stageIdx << " weak=" << r << " feature=" << wk.featureIdx
                      << " err=" << wk.err << " alpha(C)=" << wk.alpha << " parity=" << static_cast<int>(wk.parity)
                      << " hit=" << cal.hitRate << " fa=" << cal.falseAlarm << " negSurvive=" << cal.negSurvive << "/"
                      << numNeg << "\n";
            if (cal.satisfied) {
                satisfied = true;
                break;
            }
        }
        const int stageTrees = static_cast<int>(weaks.size()) - stageFirst;
        if (stageTrees <= 0) {
            std::cerr << "[WARN] Stage " << stageIdx << " produced no weak classifiers, stop\n";
            break;
        }
        // negatives the stage keeps (UpdateActiveNegByThresholdKernel, main.cu:960-983)
        std::vector<float> strong(static_cast<size_t>(n));
        if (!cuda_ok(cudaMemcpy(strong.data(), dStrong.p, sizeof(float) * n, cudaMemcpyDeviceToHost), "strong"))
            return 1;
        int remainNeg = 0;
        for (int i = numPos; i < n; ++i) remainNeg += strong[i] >= stageThreshold ? 1 : 0;
        const float totalFalseAlarm = static_cast<float>(remainNeg) / static_cast<float>(numNeg);
        if (!satisfied && remainNeg > 0) {
            std::cerr << "[WARN] Stage " << stageIdx << " did not meet target (hit>=" << minHitRate
                      << ", fa<=" << maxFalseAlarm << "). Increase maxWeakPerStage or improve training data.\n";
            break;
        }
        stages.push_back(vj_cascade_stage{stageFirst, stageTrees, stageThreshold - 1e-5f});
        std::cout << "[TRAIN] Stage " << stageIdx << " done: ntrees=" << stageTrees << " threshold=" << stageThreshold
                  << " stageOK=" << (satisfied ? 1 : 0) << " remainNeg=" << remainNeg << "/" << numNeg
                  << " totalFA=" << totalFalseAlarm << "\n";
        if (remainNeg == 0) break;
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    std::cout << "[TRAIN] elapsed(ms): " << std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count()
              << "\n";
    vj_detector_destroy(miner);
    vj_trainer_destroy(tr);
    if (weaks.empty() || stages.empty()) {
        std::cerr << "[ERR] no trained cascade stages\n";
        return 1;
    }
    std::vector<vj_stump4> stumps(weaks.size());
    for (size_t i = 0; i < weaks.size(); ++i) {
        float fb;
        std::memcpy(&fb, &weaks[i].featureIdx, 4);
        stumps[i] = vj_stump4{fb, weaks[i].theta, weaks[i].leftVal, weaks[i].rightVal};
    }
    if (vj_model_save(modelOutPath.c_str(), kWin, kWin, feats.data(), nf, stumps.data(),
                      static_cast<int64_t>(stumps.size()), stages.data(), static_cast<int64_t>(stages.size())) != VJ_OK) {
        std::cerr << "[ERR] saveCascadeModel failed: " << modelOutPath << "\n";
        return 1;
    }
    std::cout << "[OK] Saved model to: " << modelOutPath << " (features=" << nf << ", stumps=" << stumps.size()
              << ", stages=" << stages.size() << ")\n";
    return 0;
}
