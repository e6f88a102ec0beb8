/*
 * vjgb.h - C ABI of the GB300-native Viola-Jones data-parallel path.
 *
 * The reference (hengyizhu/CS677s26) exposes this path as two C++ classes,
 * vj::FaceVisionEngine (include/vj/face_vision_engine.cuh:19-196) and
 * vj::AdaBoostTrainer (include/vj/boosting_core.cuh:20-161), plus
 * vj::ModelIO (include/vj/model_io.hpp:10-20) and the `cuda_hello train|detect`
 * CLI (src/main.cu:1370-2579).  Every entry point below replaces one of those
 * members; the comment on each names the member it replaces.
 *
 * Conventions
 *  - Every function returns an int status with the numeric values of
 *    vj::Status (include/vj/common_types.cuh:11-17).  Nothing throws across
 *    the ABI.  vj_last_error() returns a message for the calling thread.
 *  - Pointers named d_* are device pointers; h_* / unprefixed are host
 *    pointers.  `stream` is a cudaStream_t passed as void* (NULL = legacy
 *    default stream), as in the reference's optional stream arguments.
 *  - The POD structs have the same size, field order and byte layout as the
 *    reference's (common_types.cuh:26-143), so cascade_model.bin files and
 *    detection arrays are interchangeable.
 *  - Handles are not thread-safe (like the reference classes); use one handle
 *    per thread.  The serving loop (vj_server_*) owns its own threads.
 */
#ifndef VJGB_H
#define VJGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__cplusplus)
#define VJ_ALIGN16 alignas(16)
#else
#define VJ_ALIGN16 _Alignas(16)
#endif

/* vj::Status, include/vj/common_types.cuh:11-17 */
enum {
    VJ_OK = 0,
    VJ_INVALID_ARG = 1,
    VJ_CUDA_ERROR = 2,
    VJ_OUT_OF_MEMORY = 3,
    VJ_RUNTIME_ERROR = 4
};

/* FaceVisionEngine::FeatureMode, include/vj/face_vision_engine.cuh:24 */
enum { VJ_FEATURES_BASIC = 0, VJ_FEATURES_CORE = 1, VJ_FEATURES_ALL = 2 };

/* Window variance normalisation used by detection.
 * VJ_NORM_FLOAT_CORNERS: the window sum is formed from float-cast integral
 *   corners, as the reference GPU kernel does (src/face_vision_engine.cu:484).
 * VJ_NORM_EXACT_INT: the window sum is an exact integer difference, as the
 *   reference CPU path does (src/main.cu:768-771).
 * Both use the unsigned 32-bit squared-sum delta (face_vision_engine.cu:475-478). */
enum { VJ_NORM_FLOAT_CORNERS = 0, VJ_NORM_EXACT_INT = 1 };

/* vj::FastRect, common_types.cuh:26-35 (20 bytes) */
typedef struct {
    int32_t p0, p1, p2, p3;
    float w;
} vj_fast_rect;

/* vj::HaarFeature, common_types.cuh:37-46 (64 bytes) */
typedef struct {
    vj_fast_rect r0, r1, r2;
    uint8_t rectCount;
    uint8_t tilted;
    uint16_t reserved;
} vj_haar_feature;

/* vj::GpuStump4, common_types.cuh:138-143 (16 bytes, 16-aligned):
 * {featureIdx as int bits, theta, leftVal, rightVal} */
typedef struct {
    VJ_ALIGN16 float featureBits;
    float theta;
    float leftVal;
    float rightVal;
} vj_stump4;

/* vj::CascadeStage, common_types.cuh:117-123 (12 bytes) */
typedef struct {
    int32_t first;
    int32_t ntrees;
    float threshold;
} vj_cascade_stage;

/* vj::Detection, common_types.cuh:126-136 (24 bytes) */
typedef struct {
    int32_t x, y, w, h, scaleIdx;
    float score;
} vj_detection;

/* vj::FeatureBestSplit, common_types.cuh:84-91 (16 bytes) */
typedef struct {
    float bestErr;
    float bestTheta;
    int32_t bestSplitPos;
    int8_t bestParity;
    int8_t pad0, pad1, pad2;
} vj_feature_best_split;

/* vj::TileBestCandidate, common_types.cuh:93-100 (16 bytes) */
typedef struct {
    float bestErr;
    float bestTheta;
    int32_t featureIdx;
    int8_t bestParity;
    int8_t pad0, pad1, pad2;
} vj_tile_best;

/* vj::WeakClassifier, common_types.cuh:102-115 (28 bytes) */
typedef struct {
    int32_t featureIdx;
    float theta;
    int8_t parity;
    int8_t pad0, pad1, pad2;
    float err;
    float alpha;
    float leftVal;
    float rightVal;
} vj_weak_classifier;

/* Message describing the last non-VJ_OK status returned on this thread. */
const char* vj_last_error(void);

/* Library build identification (compute capability the kernels target). */
const char* vj_build_info(void);

/* Per-kernel timing (no reference counterpart; the reference times whole calls
 * with cudaEvents in its compare modes, src/main.cu:1157-1188).  While enabled,
 * every kernel launch of this library is bracketed by CUDA events on its
 * stream; vj_profile_read synchronises on them and returns, per kernel name,
 * the launch count and summed device time, optionally clearing the records. */
typedef struct {
    char name[48];
    int64_t launches;
    double total_ms;
} vj_profile_entry;

int vj_profile_enable(int on);
int vj_profile_read(vj_profile_entry* out, int capacity, int* count, int reset);

/* ------------------------------------------------------------------------ */
/* Feature pool                                                             */
/* ------------------------------------------------------------------------ */

/* FaceVisionEngine::countHaarFeatures, face_vision_engine.cu:877-880 */
int vj_feature_pool_count(int mode, int winW, int winH, int64_t* count);

/* FaceVisionEngine::buildHaarFeaturePool, face_vision_engine.cu:882-1020.
 * Same enumeration order (x, y, dx, dy, type), so featureIdx values agree. */
int vj_feature_pool_build(int mode, int winW, int winH, vj_haar_feature* out,
                          int64_t capacity, int64_t* count);

/* ------------------------------------------------------------------------ */
/* Model file (cascade_model.bin)                                           */
/* ------------------------------------------------------------------------ */

/* ModelIO::saveCascadeModel, src/model_io.cpp:66-115.  Byte-identical file:
 * [48 B header "VJCBIN1\0" v1][HaarFeature x F][GpuStump4 x S][CascadeStage x K] */
int vj_model_save(const char* path, int winW, int winH,
                  const vj_haar_feature* features, int64_t featureCount,
                  const vj_stump4* stumps, int64_t stumpCount,
                  const vj_cascade_stage* stages, int64_t stageCount);

/* First half of ModelIO::loadCascadeModel (src/model_io.cpp:117-160): reads
 * and validates the header, returns the array sizes. */
int vj_model_load_header(const char* path, int* winW, int* winH,
                         int64_t* featureCount, int64_t* stumpCount,
                         int64_t* stageCount);

/* ModelIO::loadCascadeModel, src/model_io.cpp:117-167.  Arrays must hold the
 * counts returned by vj_model_load_header. */
int vj_model_load(const char* path, vj_haar_feature* features, int64_t featureCap,
                  vj_stump4* stumps, int64_t stumpCap,
                  vj_cascade_stage* stages, int64_t stageCap);

/* ------------------------------------------------------------------------ */
/* Integral images                                                          */
/* ------------------------------------------------------------------------ */

/* FaceVisionEngine::computeIntegralBatchTransposed (face_vision_engine.cu:
 * 1057-1158) for training batches.  d_gray holds n images of w x h at row
 * stride `stride`, image after image (image pitch h*stride).  Outputs use the
 * transposed layout [(h+1)*(w+1)][n]: d_sumT uint32, d_sqsumT uint64 (exact;
 * its low 32 bits are the reference's int32 bits), d_invNorm float[n]
 * (face_vision_engine.cu:216-259).  d_sqsumT and d_invNorm may be NULL. */
int vj_integral_batch(const uint8_t* d_gray, int w, int h, int stride, int n,
                      uint32_t* d_sumT, uint64_t* d_sqsumT, float* d_invNorm,
                      void* stream);

/* Single image, row-major (h+1) x (w+1) layout: the N=1 path of
 * computeIntegralBatchTransposed (face_vision_engine.cu:1109-1120) that
 * detection uses.  d_sqsum may be NULL. */
int vj_integral_image(const uint8_t* d_gray, int w, int h, int stride,
                      uint32_t* d_sum, uint64_t* d_sqsum, void* stream);

/* vj_integral_image for callers that must not allocate device memory (no
 * counterpart in the reference).  Some callers cannot call cudaMalloc: code
 * running under a caller-owned memory pool or a fixed device-memory budget,
 * and code that must not trigger the implicit synchronisation or the failure
 * paths of the CUDA allocator in the middle of a latency-bound pipeline.
 * This variant allocates nothing: its scratch (the column-pass segment totals
 * and the job descriptor, about 3.2 MB) is a fixed array in device memory that
 * every GPU loading the library holds until the process exits.  Limits:
 * w <= 3840, h <= 2160, and d_sqsum must be given (there is no room for
 * temporary squared sums); larger inputs return VJ_INVALID_ARG.  The first
 * call on each device (and the first after that device's context was reset
 * and created again) looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * Every call shares the
 * one array: calls that overlap on the GPU (different streams, or different
 * host threads) race and corrupt each other's results; keep them on one
 * stream.  Asynchronous on `stream`; results equal vj_integral_image's. */
int vj_integral_image_noalloc(const uint8_t* d_gray, int w, int h, int stride,
                              uint32_t* d_sum, uint64_t* d_sqsum, void* stream);

/* ------------------------------------------------------------------------ */
/* AdaBoost stump search (vj::AdaBoostTrainer)                              */
/* ------------------------------------------------------------------------ */

typedef struct vj_trainer vj_trainer;

/* AdaBoostTrainer::AdaBoostTrainer, boosting_core.cu:465-559.  maxSamples is
 * limited to 65535 as in the reference (16-bit sample indices,
 * boosting_core.cu:704). */
int vj_trainer_create(int winW, int winH, int maxSamples, vj_trainer** out);
int vj_trainer_destroy(vj_trainer* t);

/* FaceVisionEngine::uploadFeaturePool (face_vision_engine.cu:1022-1055) for
 * the training pool; host array, copied to the device.  Tilted features are
 * evaluated as the reference evaluates them: their four corner indices on the
 * upright integral (the reference builds no tilted integral). */
int vj_trainer_set_features(vj_trainer* t, const vj_haar_feature* features,
                            int64_t count);

/* AdaBoostTrainer::bindTrainingSet, boosting_core.cu:684-745.  Non-owning
 * device views: transposed sums [625][n] (uint32), invNorm[n], labels (+1/-1),
 * active mask (NULL = all active), weights (float, updated in place by
 * vj_round_update). */
int vj_trainer_bind(vj_trainer* t, const uint32_t* d_sumT, const float* d_invNorm,
                    int n, const int8_t* d_label, const uint8_t* d_active,
                    float* d_weight);

/* AdaBoostTrainer::evaluateFeatureResponses, boosting_core.cu:747-787.
 * d_out is [featureCount][n] float (the reference's response layout). */
int vj_trainer_evaluate_responses(vj_trainer* t, int featureBegin, int featureCount,
                                  float* d_out, void* stream);

/* AdaBoostTrainer::sortSamplesPerFeature, boosting_core.cu:829-892: stable
 * ascending sort of each feature row, -0.0f before +0.0f (radix float order);
 * d_sortedIdx is [featureCount][n] uint16. */
int vj_trainer_sort_per_feature(vj_trainer* t, const float* d_resp, int featureCount,
                                uint16_t* d_sortedIdx, void* stream);

/* AdaBoostTrainer::evaluateAndFindThreshold, boosting_core.cu:789-827.  Best
 * split per feature with compensated (Kahan) FP32 prefix sums; tie-break
 * err, then split, then parity +1 (boosting_core.cu:59-79). */
int vj_trainer_find_thresholds(vj_trainer* t, const float* d_resp,
                               const uint16_t* d_sortedIdx, int featureCount,
                               vj_feature_best_split* d_out, void* stream);

/* AdaBoostTrainer::selectBestInTile, boosting_core.cu:894-925: skips features
 * whose used-mask byte is set; ties go to the lower featureIdx. */
int vj_trainer_select_best_in_tile(vj_trainer* t, const vj_feature_best_split* d_best,
                                   int featureBegin, int featureCount,
                                   const uint8_t* d_usedMask, vj_tile_best* d_out,
                                   void* stream);

/* Stage gate (no reference counterpart): d_gate is a device int (or NULL to
 * turn gating off).  While it is nonzero, vj_stump_search, vj_round_update and
 * vj_stage_calibrate launch kernels that return at once.  vj_round_update sets
 * it to 2 when the search found no valid stump (nothing is updated, no weak
 * classifier is written); vj_stage_calibrate sets it to 1 when the stage meets
 * its targets (hit >= minHitRate and false alarm <= maxFalseAlarm, or no
 * negative survives).  A caller zeroes it, queues a stage's rounds (or chunks
 * of them) without reading anything back between them, and reads the gate and
 * the per-round records afterwards - the reference's stage loop
 * (main.cu:2005-2166) without a host round trip per round. */
int vj_trainer_set_stage_gate(vj_trainer* t, int* d_gate);

/* One boosting round's full best-weak search over the whole pool: the tile
 * loop of src/main.cu:2013-2053 plus ReduceTileBestCandidatesKernel
 * (main.cu:999-1028), fused.  The returned stump (feature, threshold, parity,
 * FP32 error) is the one the reference's CPU search runCpuWeakSearch
 * (main.cu:587-682) returns for the same weights, with the used mask applied.
 * If vj_trainer_prepare_stage was called after the last bind, the resident
 * per-feature sample orders are used instead of re-sorting.  d_out is device
 * memory (vj_tile_best[1]); nothing is copied to the host. */
int vj_stump_search(vj_trainer* t, const uint8_t* d_usedMask, vj_tile_best* d_out,
                    void* stream);

/* Evaluate and sort every feature once and keep the per-feature sample
 * orders resident on the device (2 B per feature-sample) for the rounds of
 * the current stage.  Invalidated by vj_trainer_bind. */
int vj_trainer_prepare_stage(vj_trainer* t, void* stream);

/* Restricts vj_trainer_prepare_stage and vj_stump_search to the features
 * [featureBegin, featureBegin + featureCount) of the pool: one feature tile
 * of the reference's round loop (main.cu:2013-2053, the begin/count of each
 * evaluateFeatureResponses .. selectBestInTile pass), kept for every round.
 * The search's featureIdx and the used mask stay indexed by the whole pool,
 * and vj_round_update still applies any feature of the pool, so ranks that
 * each own one range exchange their 16-byte candidates, reduce them with
 * vj_reduce_tile_best and apply the same update.  Setting a new pool resets
 * the range to the whole pool; changing it invalidates prepared orders. */
int vj_trainer_set_search_range(vj_trainer* t, int64_t featureBegin, int64_t featureCount);

/* ReduceTileBestCandidatesKernel (main.cu:991-1028): d_out = the best of
 * count candidates (device arrays), lower FP32 error first, then lower
 * featureIdx; a candidate with featureIdx -1 (no valid split) wins only when
 * every candidate has none. */
int vj_reduce_tile_best(const vj_tile_best* d_in, int count, vj_tile_best* d_out, void* stream);

/* Statistics of the last vj_stump_search (no reference counterpart): the
 * fast-pass minimum error, the width of the candidate window, how many
 * features were replayed exactly, the active weight totals, and the two
 * smallest exact (reference-replayed FP32) errors among the candidates - the
 * pick and its runner-up (runnerUpFeature -1 and runnerUpErr +inf when the pick
 * was the only candidate: every other feature's fast error exceeded the pick's
 * by more than the window).  `swept` counts the features whose orders the
 * search streamed: from the second round of a stage on, features whose error
 * bound shows they cannot reach the candidate window are skipped (the pick is
 * unchanged; bounds are used only while the weights change by
 * vj_round_update alone).  Copies from the device after synchronising. */
typedef struct {
    float fastMin;
    float window;
    int32_t candidates;
    int32_t status;  /* 0 ok, 1 no valid split in any feature */
    float totalPos;
    float totalNeg;
    float bestErr;
    int32_t bestFeature;
    float runnerUpErr;
    int32_t runnerUpFeature;
    int32_t swept;       /* features the sweep streamed (the others were pruned or used) */
    int32_t pad0;
    int64_t sweptTotal;  /* features streamed by every search of this trainer so far */
} vj_round_info;

int vj_trainer_last_round(vj_trainer* t, vj_round_info* out);

/* Resident memory used by vj_trainer_prepare_stage for n samples, in bytes. */
int vj_trainer_stage_bytes(vj_trainer* t, int n, int64_t* bytes);

/* AdaBoost round update, src/main.cu:2082-2166 with the kernels at
 * main.cu:829-906: clamp err to [1e-6, 1-1e-6], C = log((1-e)/e) (FP64 on the
 * device), leaves (parity>0: left=-C, right=+C), strong[i] += leaf, weights of
 * misclassified active samples *= exp(C), inactive weights = 0, renormalise to
 * sum 1 (FP64, exact sums).  d_best comes from vj_stump_search; d_weak_out
 * (device, may be NULL) receives the WeakClassifier; d_usedMask (may be NULL)
 * gets the chosen feature marked. */
int vj_round_update(vj_trainer* t, const vj_tile_best* d_best, float* d_strong,
                    uint8_t* d_usedMask, vj_weak_classifier* d_weak_out, void* stream);

/* Result of the stage calibration of src/main.cu:2168-2300. */
typedef struct {
    float cutVal;          /* sorted positive score at cutIdx */
    float stageThreshold;  /* cut or nextafter(cut, +inf) */
    int32_t strictGt;      /* 1 if '>' was chosen */
    int32_t posPass;
    int32_t negSurvive;
    float hitRate;
    float falseAlarm;
    int32_t satisfied;     /* (hit >= minHit && fa <= maxFA) || negSurvive == 0 */
} vj_stage_calib;

/* Stage calibration after a round, src/main.cu:2168-2300: positives are
 * samples [0, numPos).  d_out is device memory. */
int vj_stage_calibrate(vj_trainer* t, const float* d_strong, int numPos,
                       float minHitRate, float maxFalseAlarm, int stageNegBaseCount,
                       vj_stage_calib* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Multiscale detection (vj::FaceVisionEngine detect side)                  */
/* ------------------------------------------------------------------------ */

typedef struct vj_detector vj_detector;

/* FaceVisionEngine::FaceVisionEngine for detection (face_vision_engine.cu:
 * 644-725): buffers for images up to maxImageW x maxImageH and maxDetections
 * raw detections. */
int vj_detector_create(int winW, int winH, int maxImageW, int maxImageH,
                       int maxDetections, vj_detector** out);
int vj_detector_destroy(vj_detector* d);

/* FaceVisionEngine::setCascadeModel, face_vision_engine.cu:1176-1354.  Host
 * arrays; the model is copied and decoded into a compact per-stump layout.
 * Stumps must reference features in [0, featureCount). */
int vj_detector_set_model(vj_detector* d, const vj_haar_feature* features,
                          int64_t featureCount, const vj_stump4* stumps,
                          int64_t stumpCount, const vj_cascade_stage* stages,
                          int64_t stageCount);

/* FaceVisionEngine::clearCascadeModel, face_vision_engine.cu:1356-1399 */
int vj_detector_clear_model(vj_detector* d);

/* Selects the window-normalisation arithmetic (VJ_NORM_*); default
 * VJ_NORM_FLOAT_CORNERS (the reference GPU kernel's). */
int vj_detector_set_norm_mode(vj_detector* d, int mode);

/* FaceVisionEngine::detectMultiScale, face_vision_engine.cu:1541-1747.
 * image is a host pointer unless image_on_device != 0.  Raw detections are
 * returned in canonical order (pyramid level, then y, then x), the order of
 * the reference's CPU path (main.cu:765-818), the first maxDetections of them.
 * With applyGrouping the groupRectangles step (eps 0.2,
 * face_vision_engine.cu:1401-1539) runs on the device over that list: the
 * clusters, their averages, scores and scaleIdx and the containment filter
 * are the reference's; the clusters come out ordered by the canonical position
 * of their first member (the reference's own order follows its raw
 * detections' atomic order).  `out` is a host array of `capacity` entries;
 * *count receives the number written.  Blocks until the result is on the
 * host, like the reference. */
int vj_detect(vj_detector* d, const uint8_t* image, int w, int h, int stride,
              int image_on_device, float scaleFactor, int minNeighbors,
              int minObjectSize, int maxDetections, int applyGrouping,
              vj_detection* out, int capacity, int* count, void* stream);

/* FaceVisionEngine::groupRectanglesCpu (face_vision_engine.cu:1401-1539) on
 * the host, with the reference's cluster order for the given input order,
 * exposed so raw detections can be grouped separately (vj_detect groups on
 * the device).  out needs room for n entries. */
int vj_group_rectangles(const vj_detection* in, int n, int minNeighbors, float eps,
                        vj_detection* out, int* count);

/* cropResizeTo24 (main.cu:245-284), the hard-negative miner's crop, on the
 * device for many windows: crop k is the rectangle (x, y, w, h) of boxes[k]
 * (a Detection; max(1, w) by max(1, h), clamped at the border) of image
 * imageOf[k], resized with pixel-centre bilinear interpolation to
 * outSize x outSize bytes at d_out + k * outSize * outSize (outSize 24 is the
 * reference's).  images[i] are device pointers of w[i] x h[i] pixels with row
 * stride stride[i]; the other arrays are host arrays.  Asynchronous on the
 * stream. */
int vj_crop_resize_batch(int nImages, const uint8_t* const* images, const int* w, const int* h,
                         const int* stride, int nCrops, const int* imageOf, const vj_detection* boxes,
                         int outSize, uint8_t* d_out, void* stream);

/* Batched detection of n images in one pass (no reference counterpart; each
 * image's result equals vj_detect on that image alone).  All pyramid levels of
 * all images are scanned by one persistent kernel launch, replayed from a
 * captured CUDA graph.  Images are host pointers unless images_on_device.
 * Host images are read before the call returns: a page-locked image whose
 * stride is a multiple of 16 is copied as one block; the others, when they
 * add up to 16 MB or more, are first gathered by host threads into a pinned
 * buffer of the detector, else copied row by row.
 * out holds n * capPerImage entries (image i at out + i*capPerImage); counts[i]
 * receives image i's count. */
int vj_detect_batch(vj_detector* d, int n, const uint8_t* const* images,
                    const int* w, const int* h, const int* stride,
                    int images_on_device, float scaleFactor, int minNeighbors,
                    int minObjectSize, int maxDetectionsPerImage, int applyGrouping,
                    vj_detection* out, int capPerImage, int* counts, void* stream);

/* Work counts and phase times of the last vj_detect / vj_detect_batch call on
 * a detector (no reference counterpart; the windows/s and stumps/s figures of
 * a run). */
typedef struct vj_detect_stats {
    int64_t images;          /* images in the call */
    int64_t levels;          /* pyramid levels scanned */
    int64_t pyramidPixels;   /* pixels of every scanned level */
    int64_t windows;         /* window positions on the levels' scan grids */
    int64_t gated;           /* windows through the variance gate */
    int64_t stumpEvals;      /* stump evaluations */
    int64_t rawDetections;   /* windows through every stage, before truncation */
    int64_t deepWindows;     /* windows entering the warp-per-window deep pass */
    int32_t attempts;        /* 1, or more when a work buffer had to grow */
    int32_t queuePasses;     /* lane-per-window queue passes after the tile pass */
    double gpuMs;            /* device time of the detection launch */
    double phaseMs[7];       /* pyramid, integrals, tile pass, queue passes,
                                deep pass, grouping, output to the host buffer */
    double hostMs[3];        /* host wall time: planning and upload, waiting
                                for the device, sorting raw detections or
                                copying grouped ones */
} vj_detect_stats;

int vj_detector_last_stats(const vj_detector* d, vj_detect_stats* out);

/* Failure-path test of the detection kernel's grid barrier (no reference
 * counterpart): while holdBlock >= 0, that block of the next launches leaves
 * the kernel before the first barrier, and the other blocks' wait for it runs
 * out after timeoutNs (0 = the normal 60 s limit); the call then returns
 * VJ_RUNTIME_ERROR and the context stays usable.  holdBlock -1 restores
 * normal launches. */
int vj_detector_test_barrier_timeout(vj_detector* d, int holdBlock, int64_t timeoutNs);

/* Launch shape of the detection kernel (no reference counterpart).  Every
 * configuration gives the same detections; they differ only in speed. */
typedef struct vj_detect_config {
    int32_t tileRows;     /* rows of the 32-wide window tile a warp scans in
                             the tile pass: 4, 8 or 16 */
    int32_t tileStumps;   /* the tile pass runs whole stages until it has
                             covered at least this many stumps */
    int32_t queueStumps;  /* lane-per-window queue passes then cover at least
                             this many more stumps (0 = none) before the
                             warp-per-window deep pass takes the rest */
    int32_t blocksPerSM;  /* persistent CTAs per SM (0 = as many as fit); 4 or
                             more selects the kernel compiled for 4 CTAs per
                             SM (64 registers per thread) */
    int32_t deepSlots;    /* windows a warp holds in the deep pass: 1 or 2 (1 halves
                             the deep pass's shared memory, leaving more L1) */
    int32_t reserved;     /* 0 */
} vj_detect_config;

int vj_detector_set_config(vj_detector* d, const vj_detect_config* cfg);
int vj_detector_get_config(const vj_detector* d, vj_detect_config* cfg);

/* Reserves one device arena of `bytes` for the detector's work buffers (0 =
 * back to buffers grown on demand).  Every batch is then laid out inside it,
 * the queues taking what the other buffers leave; a batch that does not fit
 * returns VJ_OUT_OF_MEMORY.  The serving loop reserves each worker's share of
 * its HBM budget this way. */
int vj_detector_reserve(vj_detector* d, int64_t bytes);

/* CTAs per SM the detection kernel can keep resident with the current
 * config's tile rows (the ceiling for blocksPerSM). */
int vj_detector_occupancy(vj_detector* d, int* blocksPerSM);

/* Device bytes the detector's work buffers hold now. */
int vj_detector_device_bytes(const vj_detector* d, int64_t* bytes);

/* Upper estimate of the device bytes one w x h image adds to a batch
 * (image copy, pyramid levels, integral images, queue and detection space);
 * the serving loop admits requests against its HBM budget with it. */
int vj_detect_estimate_bytes(int winW, int winH, int w, int h, float scaleFactor,
                             int minObjectSize, int maxDetections, int64_t* bytes);

/* Autotuner: runs every candidate configuration on the given images
 * (vj_detect_batch arguments, without grouping), `repeats` timed launches
 * each, checks that each candidate's raw detections equal the first
 * candidate's, and keeps the fastest on the detector.  *chosen and *chosenMs
 * (median device ms of the winner) may be null. */
int vj_detector_autotune(vj_detector* d, int n, const uint8_t* const* images,
                         const int* w, const int* h, const int* stride,
                         int images_on_device, float scaleFactor, int minObjectSize,
                         int repeats, vj_detect_config* chosen, double* chosenMs);

/* ------------------------------------------------------------------------ */
/* Serving loop (no reference counterpart; the reference detects one image  */
/* per call, src/main.cu:2394-2579).                                        */
/*                                                                          */
/* Requests of any size are queued as they arrive.  Each worker owns a      */
/* detector and a CUDA stream; when a worker is free it takes every queued  */
/* request that fits its share of the HBM budget (by                        */
/* vj_detect_estimate_bytes) and runs them as one vj_detect_batch launch,   */
/* so requests arriving while other batches are on the GPU join the next    */
/* one (continuous batching).  With blocksPerSM 0 each worker's kernel      */
/* fills the GPU and the workers' kernels take turns on the device (one     */
/* worker's planning, uploads and copies overlap another's kernel); a       */
/* smaller blocksPerSM splits the SMs and lets batches run side by side.    */
/* maxBatchPixels caps a batch's work.  Every result equals vj_detect on    */
/* that image alone.                                                        */
/* ------------------------------------------------------------------------ */

typedef struct vj_server vj_server;

typedef struct vj_server_config {
    int32_t winW, winH;            /* model window */
    int32_t maxImageW, maxImageH;  /* largest request image */
    int32_t workers;               /* in-flight batches (>= 1) */
    int32_t maxBatchImages;        /* images per batch at most (1 = plain per-image detect) */
    int64_t hbmBudgetBytes;        /* device bytes for all in-flight batches */
    float scaleFactor;             /* detectMultiScale arguments for every request */
    int32_t minNeighbors;
    int32_t minObjectSize;
    int32_t maxDetections;
    int32_t applyGrouping;
    int32_t blocksPerSM;           /* persistent CTAs per SM per worker; 0 = all that fit,
                                      with the workers' kernels taking turns on the device */
    int32_t tileRows;              /* launch shape (vj_detect_config); 0 = default */
    int32_t tileStumps;
    int64_t maxBatchPixels;        /* pixels per batch at most (a lone larger image still
                                      runs); 0 = no limit */
} vj_server_config;

typedef struct vj_server_stats {
    int64_t submitted, completed, failed, batches;
    double meanBatchImages;
    double meanMs, p50Ms, p99Ms, p999Ms, maxMs;  /* latency: submit to result ready */
    double elapsedS;                            /* first submit to last completion */
    double imagesPerS;                          /* completed / elapsedS */
    int64_t peakAdmittedBytes;                  /* high-water mark of admitted estimates */
    int64_t deviceBytes;                        /* work buffers the workers' detectors hold */
} vj_server_stats;

/* Copies the model (as vj_detector_set_model) and starts the workers. */
int vj_server_create(const vj_server_config* cfg, const vj_haar_feature* features,
                     int64_t featureCount, const vj_stump4* stumps, int64_t stumpCount,
                     const vj_cascade_stage* stages, int64_t stageCount, vj_server** out);

/* Queues a host image (copied; the caller may reuse its buffer at once) and
 * returns a ticket.  VJ_OUT_OF_MEMORY if the image alone exceeds a worker's
 * share of the budget. */
int vj_server_submit(vj_server* s, const uint8_t* image, int w, int h, int stride,
                     uint64_t* ticket);

/* *done = 1 once the ticket's result is ready. */
int vj_server_poll(vj_server* s, uint64_t ticket, int* done);

/* Waits up to timeoutMs (< 0: no limit) for the ticket, copies up to
 * capacity detections to out, sets *count and releases the ticket.  Returns
 * VJ_RUNTIME_ERROR on timeout (the ticket stays valid) and the batch's status
 * if its detection failed. */
int vj_server_wait(vj_server* s, uint64_t ticket, int timeoutMs, vj_detection* out,
                   int capacity, int* count);

int vj_server_get_stats(vj_server* s, vj_server_stats* out);
int vj_server_reset_stats(vj_server* s);

/* Finishes the queued requests, stops the workers and frees everything. */
int vj_server_destroy(vj_server* s);

/* ------------------------------------------------------------------------ */
/* Synthetic inputs (no reference counterpart: they stand in for the Kaggle  */
/* faces, COCO negatives and demo images the reference trains and detects   */
/* on).  Deterministic integer/IEEE arithmetic, identical on x86 and Arm.   */
/* ------------------------------------------------------------------------ */

/* nPos face-like then nNeg texture 24x24 patches, [n][24][24] uint8. */
int vj_synth_patches(uint64_t seed, int nPos, int nNeg, uint8_t* out);

/* 1/f texture scene of w x h with nPaste face patterns pasted at sizes drawn
 * log-uniformly from [minSize, maxSize]. */
int vj_synth_scene(uint64_t seed, int w, int h, int nPaste, int minSize,
                   int maxSize, uint8_t* out);

/* Synthetic cascade over the Basic pool: stage sizes 1,10,25,25,50 then the
 * rest split as evenly as possible over the remaining stages; thresholds at
 * random quantiles of feature values on synthetic patches; stage thresholds
 * at the median stage sum of texture windows reaching the stage.  stumps has
 * totalStumps entries, stages has stageCount entries. */
int vj_synth_cascade(uint64_t seed, int stageCount, int totalStumps,
                     vj_stump4* stumps, vj_cascade_stage* stages);

#ifdef __cplusplus
}
#endif

#endif /* VJGB_H */
