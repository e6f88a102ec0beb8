"""ctypes binding of libvjgb (include/vjgb.h).

This is the binding a Python caller of the C ABI uses; the structured numpy
dtypes below have the byte layouts of the reference's POD structs
(include/vj/common_types.cuh in hengyizhu/CS677s26).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libvjgb.so"

VJ_OK, VJ_INVALID_ARG, VJ_CUDA_ERROR, VJ_OUT_OF_MEMORY, VJ_RUNTIME_ERROR = range(5)
STATUS_NAMES = {0: "kOk", 1: "kInvalidArg", 2: "kCudaError", 3: "kOutOfMemory", 4: "kRuntimeError"}
FEATURES_BASIC, FEATURES_CORE, FEATURES_ALL = 0, 1, 2
NORM_FLOAT_CORNERS, NORM_EXACT_INT = 0, 1

RECT = np.dtype([("p0", "<i4"), ("p1", "<i4"), ("p2", "<i4"), ("p3", "<i4"), ("w", "<f4")])
HAAR_FEATURE = np.dtype([("r0", RECT), ("r1", RECT), ("r2", RECT), ("rectCount", "u1"),
                         ("tilted", "u1"), ("reserved", "<u2")])
STUMP4 = np.dtype([("featureBits", "<f4"), ("theta", "<f4"), ("leftVal", "<f4"), ("rightVal", "<f4")])
STAGE = np.dtype([("first", "<i4"), ("ntrees", "<i4"), ("threshold", "<f4")])
DETECTION = np.dtype([("x", "<i4"), ("y", "<i4"), ("w", "<i4"), ("h", "<i4"), ("scaleIdx", "<i4"),
                      ("score", "<f4")])
FEATURE_BEST = np.dtype([("bestErr", "<f4"), ("bestTheta", "<f4"), ("bestSplitPos", "<i4"),
                         ("bestParity", "i1"), ("pad", "i1", 3)])
TILE_BEST = np.dtype([("bestErr", "<f4"), ("bestTheta", "<f4"), ("featureIdx", "<i4"),
                      ("bestParity", "i1"), ("pad", "i1", 3)])
WEAK = np.dtype([("featureIdx", "<i4"), ("theta", "<f4"), ("parity", "i1"), ("pad", "i1", 3),
                 ("err", "<f4"), ("alpha", "<f4"), ("leftVal", "<f4"), ("rightVal", "<f4")])
STAGE_CALIB = np.dtype([("cutVal", "<f4"), ("stageThreshold", "<f4"), ("strictGt", "<i4"),
                        ("posPass", "<i4"), ("negSurvive", "<i4"), ("hitRate", "<f4"),
                        ("falseAlarm", "<f4"), ("satisfied", "<i4")])

DETECT_STATS = np.dtype([("images", "<i8"), ("levels", "<i8"), ("pyramidPixels", "<i8"), ("windows", "<i8"),
                         ("gated", "<i8"), ("stumpEvals", "<i8"), ("rawDetections", "<i8"), ("deepWindows", "<i8"),
                         ("attempts", "<i4"), ("queuePasses", "<i4"), ("gpuMs", "<f8"), ("phaseMs", "<f8", 7),
                         ("hostMs", "<f8", 3)])
DETECT_CONFIG = np.dtype([("tileRows", "<i4"), ("tileStumps", "<i4"), ("queueStumps", "<i4"), ("blocksPerSM", "<i4"),
                          ("deepSlots", "<i4"), ("reserved", "<i4")])
SERVER_CONFIG = np.dtype([("winW", "<i4"), ("winH", "<i4"), ("maxImageW", "<i4"), ("maxImageH", "<i4"),
                          ("workers", "<i4"), ("maxBatchImages", "<i4"), ("hbmBudgetBytes", "<i8"),
                          ("scaleFactor", "<f4"), ("minNeighbors", "<i4"), ("minObjectSize", "<i4"),
                          ("maxDetections", "<i4"), ("applyGrouping", "<i4"), ("blocksPerSM", "<i4"),
                          ("tileRows", "<i4"), ("tileStumps", "<i4"),
                          ("maxBatchPixels", "<i8")])
SERVER_STATS = np.dtype([("submitted", "<i8"), ("completed", "<i8"), ("failed", "<i8"), ("batches", "<i8"),
                         ("meanBatchImages", "<f8"), ("meanMs", "<f8"), ("p50Ms", "<f8"), ("p99Ms", "<f8"),
                         ("p999Ms", "<f8"), ("maxMs", "<f8"), ("elapsedS", "<f8"), ("imagesPerS", "<f8"),
                         ("peakAdmittedBytes", "<i8"), ("deviceBytes", "<i8")])
ROUND_INFO = np.dtype([("fastMin", "<f4"), ("window", "<f4"), ("candidates", "<i4"), ("status", "<i4"),
                       ("totalPos", "<f4"), ("totalNeg", "<f4"), ("bestErr", "<f4"), ("bestFeature", "<i4"),
                       ("runnerUpErr", "<f4"), ("runnerUpFeature", "<i4"), ("swept", "<i4"), ("pad0", "<i4"),
                       ("sweptTotal", "<i8")])
PHASES = ("pyramid", "integrals", "tile_pass", "queue_passes", "deep_pass", "grouping", "output")
HOST_PHASES = ("plan_upload", "wait", "post")

assert DETECT_STATS.itemsize == 160 and DETECT_CONFIG.itemsize == 24
assert SERVER_CONFIG.itemsize == 72 and SERVER_STATS.itemsize == 112 and ROUND_INFO.itemsize == 56
assert HAAR_FEATURE.itemsize == 64 and STUMP4.itemsize == 16 and STAGE.itemsize == 12
assert DETECTION.itemsize == 24 and TILE_BEST.itemsize == 16 and WEAK.itemsize == 28

vp = C.c_void_p
i32 = C.c_int
i64 = C.c_int64
u64 = C.c_uint64
f32 = C.c_float
pi32 = C.POINTER(C.c_int)
pi64 = C.POINTER(C.c_int64)
cstr = C.c_char_p

# name -> (restype, argtypes); every function declared in include/vjgb.h.
SIGNATURES = {
    "vj_last_error": (cstr, []),
    "vj_build_info": (cstr, []),
    "vj_profile_enable": (i32, [i32]),
    "vj_profile_read": (i32, [vp, i32, pi32, i32]),
    "vj_feature_pool_count": (i32, [i32, i32, i32, pi64]),
    "vj_feature_pool_build": (i32, [i32, i32, i32, vp, i64, pi64]),
    "vj_model_save": (i32, [cstr, i32, i32, vp, i64, vp, i64, vp, i64]),
    "vj_model_load_header": (i32, [cstr, pi32, pi32, pi64, pi64, pi64]),
    "vj_model_load": (i32, [cstr, vp, i64, vp, i64, vp, i64]),
    "vj_integral_batch": (i32, [vp, i32, i32, i32, i32, vp, vp, vp, vp]),
    "vj_integral_image": (i32, [vp, i32, i32, i32, vp, vp, vp]),
    "vj_integral_image_noalloc": (i32, [vp, i32, i32, i32, vp, vp, vp]),
    "vj_crop_resize_batch": (i32, [i32, vp, vp, vp, vp, i32, vp, vp, i32, vp, vp]),
    "vj_trainer_set_stage_gate": (i32, [vp, vp]),
    "vj_trainer_create": (i32, [i32, i32, i32, C.POINTER(vp)]),
    "vj_trainer_destroy": (i32, [vp]),
    "vj_trainer_set_features": (i32, [vp, vp, i64]),
    "vj_trainer_bind": (i32, [vp, vp, vp, i32, vp, vp, vp]),
    "vj_trainer_evaluate_responses": (i32, [vp, i32, i32, vp, vp]),
    "vj_trainer_sort_per_feature": (i32, [vp, vp, i32, vp, vp]),
    "vj_trainer_find_thresholds": (i32, [vp, vp, vp, i32, vp, vp]),
    "vj_trainer_select_best_in_tile": (i32, [vp, vp, i32, i32, vp, vp, vp]),
    "vj_stump_search": (i32, [vp, vp, vp, vp]),
    "vj_trainer_prepare_stage": (i32, [vp, vp]),
    "vj_trainer_set_search_range": (i32, [vp, i64, i64]),
    "vj_reduce_tile_best": (i32, [vp, i32, vp, vp]),
    "vj_trainer_stage_bytes": (i32, [vp, i32, pi64]),
    "vj_trainer_last_round": (i32, [vp, vp]),
    "vj_round_update": (i32, [vp, vp, vp, vp, vp, vp]),
    "vj_stage_calibrate": (i32, [vp, vp, i32, f32, f32, i32, vp, vp]),
    "vj_detector_create": (i32, [i32, i32, i32, i32, i32, C.POINTER(vp)]),
    "vj_detector_destroy": (i32, [vp]),
    "vj_detector_set_model": (i32, [vp, vp, i64, vp, i64, vp, i64]),
    "vj_detector_clear_model": (i32, [vp]),
    "vj_detector_set_norm_mode": (i32, [vp, i32]),
    "vj_detect": (i32, [vp, vp, i32, i32, i32, i32, f32, i32, i32, i32, i32, vp, i32, pi32, vp]),
    "vj_group_rectangles": (i32, [vp, i32, i32, f32, vp, pi32]),
    "vj_detect_batch": (i32, [vp, i32, vp, vp, vp, vp, i32, f32, i32, i32, i32, i32, vp, i32, vp, vp]),
    "vj_detector_last_stats": (i32, [vp, vp]),
    "vj_detector_test_barrier_timeout": (i32, [vp, i32, i64]),
    "vj_detector_set_config": (i32, [vp, vp]),
    "vj_detector_get_config": (i32, [vp, vp]),
    "vj_detector_autotune": (i32, [vp, i32, vp, vp, vp, vp, i32, f32, i32, i32, vp, vp]),
    "vj_detector_reserve": (i32, [vp, i64]),
    "vj_detector_occupancy": (i32, [vp, pi32]),
    "vj_detector_device_bytes": (i32, [vp, pi64]),
    "vj_detect_estimate_bytes": (i32, [i32, i32, i32, i32, f32, i32, i32, pi64]),
    "vj_server_create": (i32, [vp, vp, i64, vp, i64, vp, i64, C.POINTER(vp)]),
    "vj_server_submit": (i32, [vp, vp, i32, i32, i32, C.POINTER(C.c_uint64)]),
    "vj_server_poll": (i32, [vp, u64, pi32]),
    "vj_server_wait": (i32, [vp, u64, i32, vp, i32, pi32]),
    "vj_server_get_stats": (i32, [vp, vp]),
    "vj_server_reset_stats": (i32, [vp]),
    "vj_server_destroy": (i32, [vp]),
    "vj_synth_patches": (i32, [u64, i32, i32, vp]),
    "vj_synth_scene": (i32, [u64, i32, i32, i32, i32, i32, vp]),
    "vj_synth_cascade": (i32, [u64, i32, i32, vp, vp]),
}

_lib = None


class VJError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} -> {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def load() -> C.CDLL:
    """Loads libvjgb.so (built in-tree); raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def call(name: str, *args) -> None:
    """Calls a status-returning entry point; raises VJError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != VJ_OK:
        raise VJError(name, st, lib.vj_last_error().decode(errors="replace"))


def status(name: str, *args) -> int:
    """Calls an entry point and returns its status code without raising."""
    return getattr(load(), name)(*args)


def ptr(a) -> int | None:
    """Data pointer of a numpy array, a torch tensor or an int; None for None."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"cannot take a pointer of {type(a)}")
