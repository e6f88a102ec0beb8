/*
 * vj_oracle.h - CPU oracle for the Viola-Jones data-parallel path.
 *
 * TEST INFRASTRUCTURE.  This is the checker, not the product: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs
 * may load it.  It restates, in plain C, the reference's own CPU algorithms
 * (hengyizhu/CS677s26 src/main.cu and src/face_vision_engine.cu); each function
 * cites the lines it follows.  It is pinned against the reference itself:
 * tests/golden/ holds outputs of the reference's CPU functions compiled from
 * its sources (oracle/ref_harness.cu, oracle/Makefile), and
 * tests/test_oracle_golden.py checks this file against them.
 *
 * Structs below have the reference's byte layouts (include/vj/common_types.cuh).
 * Build with -ffp-contract=off: every float operation must round on its own,
 * as in the reference's x86 host build.
 */
#ifndef VJ_ORACLE_H
#define VJ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int32_t p0, p1, p2, p3; float w; } vjo_rect;
typedef struct { vjo_rect r0, r1, r2; uint8_t rectCount, tilted; uint16_t reserved; } vjo_feature;
typedef struct { float featureBits, theta, leftVal, rightVal; } vjo_stump;
typedef struct { int32_t first, ntrees; float threshold; } vjo_stage;
typedef struct { int32_t x, y, w, h, scaleIdx; float score; } vjo_det;

/* Result of one best-weak search (CpuBestWeakResult, main.cu:421-426) plus
 * the FP64 weighted error of the chosen split and the split position. */
typedef struct {
    int32_t featureIdx;
    float err;
    float theta;
    int32_t parity;
    int32_t split;
    double err64;
} vjo_best;

/* Haar pool, face_vision_engine.cu:882-1020 (mode 0 Basic, 1 Core, 2 All). */
int64_t vjo_feature_pool(int mode, int W, int H, vjo_feature* out, int64_t cap);

/* Integral and squared integral, (h+1) x (w+1) row-major, main.cu:428-455.
 * sum is the reference's int32 bits as uint32; sq is exact (the reference
 * keeps its low 32 bits). */
void vjo_integral(const uint8_t* gray, int w, int h, int stride, uint32_t* sum, uint64_t* sq);

/* Batch of n patches of 24x24 -> sums [n][625] and invNorm[n]
 * (main.cu:457-472 and face_vision_engine.cu:216-259). */
void vjo_train_integrals(const uint8_t* patches, int n, uint32_t* sums, float* invNorm);

/* Normalised training response of one feature on one patch, main.cu:476-496. */
float vjo_train_response(const vjo_feature* f, const uint32_t* sum625, float invNorm);

/* runCpuWeakSearch, main.cu:587-682, over features [0, nFeat) skipping those
 * with usedMask[f] != 0 (usedMask may be NULL), split over `threads` threads
 * (the per-feature result does not depend on the split).  weights/labels/
 * active are per sample (active may be NULL).  If perFeature is not NULL it
 * receives each feature's own best (err FLT_MAX-like +inf if no split). */
void vjo_weak_search(const vjo_feature* feats, int nFeat, const uint8_t* usedMask,
                     const uint32_t* sums, const float* invNorm, const int8_t* labels,
                     const uint8_t* active, const float* weights, int n, int threads,
                     vjo_best* out, vjo_best* perFeature);

/* Stage-resident form of vjo_weak_search.  Within a stage the responses and
 * hence every feature's sorted order stay fixed; only the weights change.
 * vjo_sorted_build sorts every feature of the pool once (6 bytes per
 * feature-sample of host memory), and vjo_sorted_search then runs the same
 * sweep and the same cross-feature rule as vjo_weak_search over the stored
 * orders, so its result equals vjo_weak_search's on the same inputs. */
typedef struct vjo_sorted vjo_sorted;
vjo_sorted* vjo_sorted_build(const vjo_feature* feats, int nFeat, const uint32_t* sums, const float* invNorm,
                             int n, int threads);
void vjo_sorted_search(const vjo_sorted* s, const uint8_t* usedMask, const int8_t* labels, const uint8_t* active,
                       const float* weights, int threads, vjo_best* out, vjo_best* perFeature);
void vjo_sorted_free(vjo_sorted* s);

/* FP64 weighted error of every feature's best split (exact-sum reference for
 * the per-round error statement).  err64[f] = +inf when the feature has no
 * valid split or is masked. */
void vjo_feature_err64(const vjo_feature* feats, int nFeat, const uint8_t* usedMask,
                       const uint32_t* sums, const float* invNorm, const int8_t* labels,
                       const uint8_t* active, const float* weights, int n, int threads,
                       double* err64);

/* One AdaBoost update with FP64 alpha/log and renormalisation, following the
 * reference's update rule (main.cu:2082-2102, 829-906) with the FP64 steps of
 * this project: C = (float)log((1-e)/e) in double; F = exp((double)C);
 * strong[i] += leaf; misclassified active weights scale by F; inactive = 0;
 * Z = sum of (double)w_i*F_i with 1024 strided sequential partials combined by
 * a fixed halving tree; w_i = (float)(w_i*F_i / Z).  Returns the weak. */
void vjo_round_update(const vjo_feature* feats, const vjo_best* best, const uint32_t* sums,
                      const float* invNorm, const int8_t* labels, const uint8_t* active,
                      float* weights, float* strong, int n, float* weakOut /* [7]:
                      theta, err, alpha, left, right, parity, featureIdx */);

/* Stage calibration, main.cu:2168-2300 (numbers in the order of
 * vj_stage_calib: cutVal, stageThreshold, strictGt, posPass, negSurvive,
 * hitRate, falseAlarm, satisfied). */
void vjo_stage_calibrate(const float* strong, const uint8_t* active, int n, int numPos,
                         float minHitRate, float maxFalseAlarm, int stageNegBase,
                         float* outF /* cut, thr, hit, fa */, int32_t* outI /* strictGt,
                         posPass, negSurvive, satisfied */);

/* resizeGrayBilinearHost, main.cu:545-585. */
void vjo_resize(const uint8_t* src, int sw, int sh, int sstride, uint8_t* dst, int dw, int dh);

/* detectMultiScaleCpu, main.cu:684-827, raw detections in scan order.
 * normMode 0: window sum from float-cast corners as the GPU kernel does
 * (face_vision_engine.cu:484); 1: exact integer sum as main.cu:768-771.
 * Returns the number of detections (at most maxDetections), written to out
 * (capacity cap).  threads > 1 splits rows of each level; the result order is
 * unchanged. */
int vjo_detect(const vjo_feature* feats, int nFeat, const vjo_stump* stumps, int nStumps,
               const vjo_stage* stages, int nStages, int winW, int winH, const uint8_t* image,
               int w, int h, int stride, float scaleFactor, int minObjectSize,
               int maxDetections, int maxScales, int normMode, int threads, vjo_det* out,
               int cap);

/* groupRectanglesCpu, face_vision_engine.cu:1401-1539.  Returns the count. */
int vjo_group(const vjo_det* in, int n, int minNeighbors, float eps, vjo_det* out);
/* cropResizeTo24 (main.cu:245-284) generalised to an out x out patch: the
 * window (x, y, bw, bh) of a w x h image with row stride `stride`, pixel-centre
 * bilinear, clamped at the image border. */
void vjo_crop_resize(const uint8_t* img, int w, int h, int stride, int x, int y, int bw, int bh, int out,
                     uint8_t* dst);

/* vjo_group with the output ordered by each cluster's first member (smallest
 * input index). */
int vjo_group_first_order(const vjo_det* in, int n, int minNeighbors, float eps, vjo_det* out);

/* Seeded synthetic inputs (vj_synth.c), byte-identical to the package's
 * generators: nPos face patterns then nNeg texture patches of 24x24; a
 * texture scene with nPaste faces at log-uniform sizes (returns 0, or -1 on
 * bad arguments); a cascade of stageCount stages and totalStumps stumps over
 * the Basic pool (returns 0 or -1). */
void vjo_synth_patches(uint64_t seed, int nPos, int nNeg, uint8_t* out);
int vjo_synth_scene(uint64_t seed, int w, int h, int nPaste, int minSize, int maxSize, uint8_t* out);
int vjo_synth_cascade(uint64_t seed, int stageCount, int totalStumps, vjo_stump* stumps, vjo_stage* stages);

#ifdef __cplusplus
}
#endif

#endif
