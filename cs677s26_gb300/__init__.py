"""GB300-native Viola-Jones data-parallel path (drop-in for hengyizhu/CS677s26).

Python mirror of the reference's C++ interface for this path, over the C ABI
of libvjgb (include/vjgb.h):

* ``FaceVisionEngine`` - vj::FaceVisionEngine (include/vj/face_vision_engine.cuh):
  ``buildHaarFeaturePool``, ``countHaarFeatures``, ``computeIntegralBatchTransposed``,
  ``setCascadeModel``, ``clearCascadeModel``, ``detectMultiScale`` (+ ``detectBatch``).
* ``AdaBoostTrainer`` - vj::AdaBoostTrainer (include/vj/boosting_core.cuh):
  ``bindTrainingSet``, ``evaluateFeatureResponses``, ``sortSamplesPerFeature``,
  ``evaluateAndFindThreshold``, ``selectBestInTile``, plus the fused round
  ``bestWeak`` and ``applyBestWeak`` (the round update of src/main.cu:2082-2166).
* ``ModelIO`` - vj::ModelIO save/load of cascade_model.bin.

Methods return ``Status`` codes like the reference (0 = kOk); constructors
raise.  Device memory is passed as torch CUDA tensors.  The CUDA library must
be built (``__graft_entry__.build()``); nothing here falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from . import _capi
from ._capi import (DETECTION, FEATURE_BEST, HAAR_FEATURE, STAGE, STAGE_CALIB, STUMP4, TILE_BEST, WEAK,
                    VJError, call, load, ptr)

__all__ = ["Status", "FeatureMode", "FaceVisionEngine", "AdaBoostTrainer", "ModelIO", "VJError", "DetectServer",
           "estimate_detect_bytes", "crop_resize_batch",
           "HAAR_FEATURE", "STUMP4", "STAGE", "DETECTION", "TILE_BEST", "WEAK", "FEATURE_BEST",
           "STAGE_CALIB", "synth_patches", "synth_scene", "synth_cascade", "feature_pool", "load"]


class Status(IntEnum):
    """vj::Status, include/vj/common_types.cuh:11-17."""
    kOk = 0
    kInvalidArg = 1
    kCudaError = 2
    kOutOfMemory = 3
    kRuntimeError = 4


class FeatureMode(IntEnum):
    """FaceVisionEngine::FeatureMode."""
    Basic = 0
    Core = 1
    All = 2


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def feature_pool(mode: int = FeatureMode.Basic, win: int = 24) -> np.ndarray:
    """Haar pool in the reference's enumeration order (HaarFeature records)."""
    n = C.c_int64()
    call("vj_feature_pool_count", int(mode), win, win, C.byref(n))
    out = np.zeros(n.value, dtype=HAAR_FEATURE)
    call("vj_feature_pool_build", int(mode), win, win, ptr(out), n.value, C.byref(n))
    return out


def synth_patches(seed: int, n_pos: int, n_neg: int) -> np.ndarray:
    """[n_pos + n_neg, 24, 24] uint8: face-like patterns, then 1/f texture."""
    out = np.empty((n_pos + n_neg, 24, 24), dtype=np.uint8)
    call("vj_synth_patches", seed, n_pos, n_neg, ptr(out))
    return out


def synth_scene(seed: int, w: int, h: int, n_paste: int = 0, min_size: int = 24, max_size: int = 300) -> np.ndarray:
    out = np.empty((h, w), dtype=np.uint8)
    call("vj_synth_scene", seed, w, h, n_paste, min_size, max_size, ptr(out))
    return out


def synth_cascade(seed: int, stages: int = 38, stumps: int = 6061):
    st = np.zeros(stumps, dtype=STUMP4)
    sg = np.zeros(stages, dtype=STAGE)
    call("vj_synth_cascade", seed, stages, stumps, ptr(st), ptr(sg))
    return st, sg


def feature_index(stumps: np.ndarray) -> np.ndarray:
    """featureIdx stored as the int bits of GpuStump4.x."""
    return stumps["featureBits"].view(np.int32)


class ModelIO:
    """vj::ModelIO, src/model_io.cpp."""

    @staticmethod
    def saveCascadeModel(path: str, win, features: np.ndarray, stumps: np.ndarray, stages: np.ndarray) -> bool:
        st = _capi.status("vj_model_save", str(path).encode(), int(win[0]), int(win[1]),
                          ptr(np.ascontiguousarray(features)), len(features),
                          ptr(np.ascontiguousarray(stumps)), len(stumps),
                          ptr(np.ascontiguousarray(stages)), len(stages))
        return st == 0

    @staticmethod
    def loadCascadeModel(path: str):
        """Returns (win, features, stumps, stages) or None if the file is invalid."""
        ww, wh = C.c_int(), C.c_int()
        nf, ns, nst = C.c_int64(), C.c_int64(), C.c_int64()
        if _capi.status("vj_model_load_header", str(path).encode(), C.byref(ww), C.byref(wh), C.byref(nf),
                        C.byref(ns), C.byref(nst)) != 0:
            return None
        f = np.zeros(nf.value, dtype=HAAR_FEATURE)
        s = np.zeros(ns.value, dtype=STUMP4)
        g = np.zeros(nst.value, dtype=STAGE)
        if _capi.status("vj_model_load", str(path).encode(), ptr(f), nf.value, ptr(s), ns.value, ptr(g),
                        nst.value) != 0:
            return None
        return (ww.value, wh.value), f, s, g


class FaceVisionEngine:
    """vj::FaceVisionEngine: integral images and multiscale detection."""

    def __init__(self, win=(24, 24), maxSamples: int = 1, maxImageW: int = 24, maxImageH: int = 24,
                 enableTilted: bool = False, maxDetections: int = 200000):
        if maxSamples <= 0 or maxImageW <= 0 or maxImageH <= 0 or maxDetections <= 0:
            raise ValueError("FaceVisionEngine: invalid constructor args")
        self.win = (int(win[0]), int(win[1]))
        self.maxSamples = maxSamples
        self.maxDetections = maxDetections
        h = C.c_void_p()
        call("vj_detector_create", self.win[0], self.win[1], maxImageW, maxImageH, maxDetections, C.byref(h))
        self._h = h
        self._iiSet = None
        self._out = None  # output records of detectMultiScale, reused between calls

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _capi.status("vj_detector_destroy", h)
            self._h = None

    @staticmethod
    def countHaarFeatures(win, mode) -> int:
        n = C.c_int64()
        call("vj_feature_pool_count", int(mode), int(win[0]), int(win[1]), C.byref(n))
        return n.value

    @staticmethod
    def buildHaarFeaturePool(win, mode) -> np.ndarray:
        return feature_pool(mode, int(win[0]))

    def computeIntegralBatchTransposed(self, dGrayBatch, imageW: int, imageH: int, imageStride: int, nSamples: int,
                                       computeInvNorm: bool = True, stream=None) -> int:
        """Integral images of a device batch; the result is kept as integralSetView()."""
        import torch
        if nSamples <= 0 or nSamples > self.maxSamples:
            return Status.kInvalidArg
        dev = dGrayBatch.device
        area = (imageW + 1) * (imageH + 1)
        sumT = torch.empty(area * nSamples, dtype=torch.int32, device=dev)
        sqT = torch.empty(area * nSamples, dtype=torch.int64, device=dev)
        inv = torch.empty(nSamples, dtype=torch.float32, device=dev) if computeInvNorm else None
        st = _capi.status("vj_integral_batch", ptr(dGrayBatch), imageW, imageH, imageStride, nSamples, ptr(sumT),
                          ptr(sqT), ptr(inv), _stream(stream))
        if st == 0:
            self._iiSet = dict(nSamples=nSamples, iiWidth=imageW + 1, iiHeight=imageH + 1, iiArea=area,
                               d_sumT=sumT, d_sqsumT=sqT, d_invNorm=inv)
        return Status(st)

    def integralSetView(self) -> dict | None:
        return self._iiSet

    def setCascadeModel(self, features: np.ndarray, stumps: np.ndarray, stages: np.ndarray) -> int:
        return Status(_capi.status("vj_detector_set_model", self._h, ptr(np.ascontiguousarray(features)),
                                   len(features), ptr(np.ascontiguousarray(stumps)), len(stumps),
                                   ptr(np.ascontiguousarray(stages)), len(stages)))

    def clearCascadeModel(self) -> int:
        return Status(_capi.status("vj_detector_clear_model", self._h))

    def setNormMode(self, mode: int) -> int:
        return Status(_capi.status("vj_detector_set_norm_mode", self._h, int(mode)))

    def detectMultiScale(self, image, imageW: int, imageH: int, imageStride: int, scaleFactor: float = 1.25,
                         minNeighbors: int = 4, minObjectSize: int = 24, maxDetections: int = 200000,
                         applyGrouping: bool = True, stream=None, capacity: int | None = None):
        """Returns (status, detections).  `image` is a host numpy array or a CUDA tensor."""
        on_dev = not isinstance(image, np.ndarray)
        cap = capacity if capacity is not None else max(1, min(maxDetections, self.maxDetections))
        if self._out is None or len(self._out) < cap:
            self._out = np.empty(cap, dtype=DETECTION)
        out = self._out
        n = C.c_int()
        st = _capi.status("vj_detect", self._h, ptr(image), imageW, imageH, imageStride, int(on_dev),
                          C.c_float(scaleFactor), minNeighbors, minObjectSize, maxDetections, int(applyGrouping),
                          ptr(out), cap, C.byref(n), _stream(stream))
        return Status(st), out[: n.value].copy()

    def detectBatch(self, images, scaleFactor: float = 1.25, minNeighbors: int = 4, minObjectSize: int = 24,
                    maxDetections: int = 200000, applyGrouping: bool = True, capPerImage: int = 4096, stream=None):
        """Detects on a list of host (numpy HxW) or device images; returns (status, [detections])."""
        n = len(images)
        on_dev = not isinstance(images[0], np.ndarray)
        ptrs = (C.c_void_p * n)(*[ptr(im) for im in images])
        ws = (C.c_int * n)(*[int(im.shape[1]) for im in images])
        hs = (C.c_int * n)(*[int(im.shape[0]) for im in images])
        ss = (C.c_int * n)(*[int(im.shape[1]) for im in images])
        out = np.zeros(n * capPerImage, dtype=DETECTION)
        cnt = np.zeros(n, dtype=np.int32)
        st = _capi.status("vj_detect_batch", self._h, n, ptrs, ws, hs, ss, int(on_dev), C.c_float(scaleFactor),
                          minNeighbors, minObjectSize, maxDetections, int(applyGrouping), ptr(out), capPerImage,
                          ptr(cnt), _stream(stream))
        res = [out[i * capPerImage: i * capPerImage + cnt[i]].copy() for i in range(n)]
        return Status(st), res

    def lastStats(self) -> dict:
        """Work counts and phase times of the last detectMultiScale / detectBatch call."""
        rec = np.zeros(1, dtype=_capi.DETECT_STATS)
        call("vj_detector_last_stats", self._h, ptr(rec))
        out = {k: rec[k][0].item() for k in _capi.DETECT_STATS.names if k not in ("phaseMs", "hostMs")}
        out["phaseMs"] = dict(zip(_capi.PHASES, [float(x) for x in rec["phaseMs"][0]]))
        out["hostMs"] = dict(zip(_capi.HOST_PHASES, [float(x) for x in rec["hostMs"][0]]))
        return out

    def reserve(self, nbytes: int) -> int:
        """Lays out every batch inside one device arena of nbytes (0 = grow on demand)."""
        return Status(_capi.status("vj_detector_reserve", self._h, int(nbytes)))

    def deviceBytes(self) -> int:
        b = C.c_int64()
        call("vj_detector_device_bytes", self._h, C.byref(b))
        return b.value

    def getConfig(self) -> dict:
        rec = np.zeros(1, dtype=_capi.DETECT_CONFIG)
        call("vj_detector_get_config", self._h, ptr(rec))
        return {k: int(rec[k][0]) for k in _capi.DETECT_CONFIG.names if k != "reserved"}

    def setConfig(self, **cfg) -> int:
        """Launch shape of the detection kernel (tileRows, tileStumps, queueStumps, blocksPerSM)."""
        cur = self.getConfig()
        cur.update(cfg)
        rec = np.zeros(1, dtype=_capi.DETECT_CONFIG)
        for k, v in cur.items():
            rec[k] = v
        return Status(_capi.status("vj_detector_set_config", self._h, ptr(rec)))

    def autotune(self, images, scaleFactor: float = 1.25, minObjectSize: int = 24, repeats: int = 2):
        """Times the candidate launch shapes on `images`, keeps the fastest; returns (status, config, ms)."""
        n = len(images)
        on_dev = not isinstance(images[0], np.ndarray)
        ptrs = (C.c_void_p * n)(*[ptr(im) for im in images])
        ws = (C.c_int * n)(*[int(im.shape[1]) for im in images])
        hs = (C.c_int * n)(*[int(im.shape[0]) for im in images])
        rec = np.zeros(1, dtype=_capi.DETECT_CONFIG)
        ms = C.c_double()
        st = _capi.status("vj_detector_autotune", self._h, n, ptrs, ws, hs, ws, int(on_dev), C.c_float(scaleFactor),
                          minObjectSize, repeats, ptr(rec), C.byref(ms))
        return Status(st), {k: int(rec[k][0]) for k in _capi.DETECT_CONFIG.names if k != "reserved"}, ms.value


def estimate_detect_bytes(w: int, h: int, scaleFactor: float = 1.25, minObjectSize: int = 24,
                          maxDetections: int = 200000, win=(24, 24)) -> int:
    """Device bytes one w x h image adds to a detection batch (admission estimate)."""
    b = C.c_int64()
    call("vj_detect_estimate_bytes", int(win[0]), int(win[1]), int(w), int(h), C.c_float(scaleFactor),
         minObjectSize, maxDetections, C.byref(b))
    return b.value


def crop_resize_batch(images, boxes, image_of, out_size: int = 24, d_out=None, stream=None):
    """cropResizeTo24 (main.cu:245-284) on the device: crop k is Detection
    boxes[k] of images[image_of[k]] (2-D uint8 CUDA tensors), resized to
    out_size x out_size.  Returns (status, patches) with patches a CUDA uint8
    tensor of shape (len(boxes), out_size, out_size)."""
    import torch
    boxes = np.ascontiguousarray(boxes, dtype=DETECTION)
    image_of = np.ascontiguousarray(image_of, dtype=np.int32)
    n = len(images)
    ptrs = (C.c_void_p * n)(*[int(im.data_ptr()) for im in images])
    ws = (C.c_int * n)(*[int(im.shape[1]) for im in images])
    hs = (C.c_int * n)(*[int(im.shape[0]) for im in images])
    ss = (C.c_int * n)(*[int(im.stride(0)) for im in images])
    if d_out is None:
        d_out = torch.empty((len(boxes), out_size, out_size), dtype=torch.uint8, device=images[0].device)
    st = _capi.status("vj_crop_resize_batch", n, ptrs, ws, hs, ss, len(boxes), ptr(image_of), ptr(boxes),
                      out_size, int(d_out.data_ptr()) if len(boxes) else None, _stream(stream))
    return Status(st), d_out


class DetectServer:
    """Continuous-batching detection server (vj_server_*): submit host images as
    they arrive, wait for each ticket's detections."""

    def __init__(self, features, stumps, stages, workers: int = 2, maxBatchImages: int = 64,
                 hbmBudgetBytes: int = 16 << 30, maxImage=(3840, 2160), scaleFactor: float = 1.25,
                 minNeighbors: int = 4, minObjectSize: int = 24, maxDetections: int = 200000,
                 applyGrouping: bool = True, blocksPerSM: int = 0, tileRows: int = 0, tileStumps: int = 0,
                 maxBatchPixels: int = 0, win=(24, 24)):
        cfg = np.zeros(1, dtype=_capi.SERVER_CONFIG)
        for k, v in dict(winW=win[0], winH=win[1], maxImageW=maxImage[0], maxImageH=maxImage[1], workers=workers,
                         maxBatchImages=maxBatchImages, hbmBudgetBytes=hbmBudgetBytes, scaleFactor=scaleFactor,
                         minNeighbors=minNeighbors, minObjectSize=minObjectSize, maxDetections=maxDetections,
                         applyGrouping=int(applyGrouping), blocksPerSM=blocksPerSM, tileRows=tileRows,
                         tileStumps=tileStumps, maxBatchPixels=maxBatchPixels).items():
            cfg[k] = v
        self._keep = [np.ascontiguousarray(a) for a in (features, stumps, stages)]
        f, s, g = self._keep
        h = C.c_void_p()
        call("vj_server_create", ptr(cfg), ptr(f), len(f), ptr(s), len(s), ptr(g), len(g), C.byref(h))
        self._h = h

    def submit(self, image: np.ndarray) -> int:
        img = np.ascontiguousarray(image, dtype=np.uint8)
        t = C.c_uint64()
        call("vj_server_submit", self._h, ptr(img), int(img.shape[1]), int(img.shape[0]), int(img.shape[1]),
             C.byref(t))
        return t.value

    def poll(self, ticket: int) -> bool:
        d = C.c_int()
        call("vj_server_poll", self._h, C.c_uint64(ticket), C.byref(d))
        return bool(d.value)

    def wait(self, ticket: int, timeoutMs: int = -1, capacity: int = 4096):
        """Returns (status, detections) and releases the ticket (unless it timed out)."""
        out = np.zeros(capacity, dtype=DETECTION)
        n = C.c_int()
        st = _capi.status("vj_server_wait", self._h, C.c_uint64(ticket), timeoutMs, ptr(out), capacity, C.byref(n))
        return Status(st), out[: n.value].copy()

    def stats(self) -> dict:
        rec = np.zeros(1, dtype=_capi.SERVER_STATS)
        call("vj_server_get_stats", self._h, ptr(rec))
        return {k: rec[k][0].item() for k in _capi.SERVER_STATS.names}

    def resetStats(self) -> None:
        call("vj_server_reset_stats", self._h)

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            _capi.status("vj_server_destroy", h)
            self._h = None

    def __del__(self):
        self.close()


class AdaBoostTrainer:
    """vj::AdaBoostTrainer: best-weak search and the AdaBoost round update."""

    def __init__(self, win=(24, 24), maxSamples: int = 20000, maxFeaturesPerTile: int = 1024):
        self.maxFeaturesPerTile = maxFeaturesPerTile
        h = C.c_void_p()
        call("vj_trainer_create", int(win[0]), int(win[1]), maxSamples, C.byref(h))
        self._h = h
        self._bound = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _capi.status("vj_trainer_destroy", h)
            self._h = None

    def setFeaturePool(self, features: np.ndarray) -> int:
        self._features = np.ascontiguousarray(features)
        return Status(_capi.status("vj_trainer_set_features", self._h, ptr(self._features), len(self._features)))

    def bindTrainingSet(self, iiSet: dict, labels, active, weights) -> int:
        """iiSet as returned by FaceVisionEngine.integralSetView(); device tensors."""
        self._bound = (iiSet, labels, active, weights)
        return Status(_capi.status("vj_trainer_bind", self._h, ptr(iiSet["d_sumT"]), ptr(iiSet["d_invNorm"]),
                                   iiSet["nSamples"], ptr(labels), ptr(active), ptr(weights)))

    def evaluateFeatureResponses(self, featureBegin: int, featureCount: int, dOutResp, stream=None) -> int:
        return Status(_capi.status("vj_trainer_evaluate_responses", self._h, featureBegin, featureCount,
                                   ptr(dOutResp), _stream(stream)))

    def sortSamplesPerFeature(self, dResp, featureCount: int, dOutSortedIdx, stream=None) -> int:
        return Status(_capi.status("vj_trainer_sort_per_feature", self._h, ptr(dResp), featureCount,
                                   ptr(dOutSortedIdx), _stream(stream)))

    def evaluateAndFindThreshold(self, dResp, dSortedIdx, featureCount: int, dOutBest, stream=None) -> int:
        return Status(_capi.status("vj_trainer_find_thresholds", self._h, ptr(dResp), ptr(dSortedIdx),
                                   featureCount, ptr(dOutBest), _stream(stream)))

    def selectBestInTile(self, dBest, featureBegin: int, featureCount: int, dUsedFeatureMask, dOut,
                         stream=None) -> int:
        return Status(_capi.status("vj_trainer_select_best_in_tile", self._h, ptr(dBest), featureBegin,
                                   featureCount, ptr(dUsedFeatureMask), ptr(dOut), _stream(stream)))

    def prepareStage(self, stream=None) -> int:
        return Status(_capi.status("vj_trainer_prepare_stage", self._h, _stream(stream)))

    def setSearchRange(self, featureBegin: int, featureCount: int) -> int:
        """Restrict prepareStage/bestWeak to one feature range of the pool (a
        rank's tile); featureIdx and the used mask stay pool-indexed."""
        return Status(_capi.status("vj_trainer_set_search_range", self._h, featureBegin, featureCount))

    def bestWeak(self, dUsedFeatureMask, dOut, stream=None) -> int:
        """One round's full search; dOut is a 16-byte device buffer (TileBestCandidate)."""
        return Status(_capi.status("vj_stump_search", self._h, ptr(dUsedFeatureMask), ptr(dOut),
                                   _stream(stream)))

    def lastRound(self) -> dict:
        """Statistics of the last bestWeak: fast minimum, window, candidates, the
        pick's and the runner-up's exact errors (vj_trainer_last_round)."""
        rec = np.zeros(1, dtype=_capi.ROUND_INFO)
        call("vj_trainer_last_round", self._h, ptr(rec))
        return {k: rec[k][0].item() for k in _capi.ROUND_INFO.names}

    def applyBestWeak(self, dBest, dStrong, dUsedFeatureMask=None, dWeakOut=None, stream=None) -> int:
        return Status(_capi.status("vj_round_update", self._h, ptr(dBest), ptr(dStrong), ptr(dUsedFeatureMask),
                                   ptr(dWeakOut), _stream(stream)))

    def calibrateStage(self, dStrong, numPos: int, minHitRate: float, maxFalseAlarm: float,
                       stageNegBaseCount: int, dOut, stream=None) -> int:
        return Status(_capi.status("vj_stage_calibrate", self._h, ptr(dStrong), numPos, C.c_float(minHitRate),
                                   C.c_float(maxFalseAlarm), stageNegBaseCount, ptr(dOut), _stream(stream)))
