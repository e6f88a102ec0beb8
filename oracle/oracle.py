"""ctypes binding of the CPU oracle (oracle/vj_oracle.c) and, where it was built,
of the reference's own CPU functions (oracle/_ref/libvjref.so).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / --impl reference legs use this module; the product path never
does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libvjref.so"

RECT = np.dtype([("p0", "<i4"), ("p1", "<i4"), ("p2", "<i4"), ("p3", "<i4"), ("w", "<f4")])
FEATURE = np.dtype([("r0", RECT), ("r1", RECT), ("r2", RECT), ("rectCount", "u1"), ("tilted", "u1"),
                    ("reserved", "<u2")])
STUMP = np.dtype([("featureBits", "<f4"), ("theta", "<f4"), ("leftVal", "<f4"), ("rightVal", "<f4")])
STAGE = np.dtype([("first", "<i4"), ("ntrees", "<i4"), ("threshold", "<f4")])
DET = np.dtype([("x", "<i4"), ("y", "<i4"), ("w", "<i4"), ("h", "<i4"), ("scaleIdx", "<i4"), ("score", "<f4")])


class Best(C.Structure):
    _fields_ = [("featureIdx", C.c_int32), ("err", C.c_float), ("theta", C.c_float), ("parity", C.c_int32),
                ("split", C.c_int32), ("err64", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


BEST = np.dtype([("featureIdx", "<i4"), ("err", "<f4"), ("theta", "<f4"), ("parity", "<i4"), ("split", "<i4"),
                 ("pad", "<i4"), ("err64", "<f8")])
assert BEST.itemsize == C.sizeof(Best)

_lib = None
_ref = None


def build(ref_src: str | None = None) -> None:
    """Builds liboracle.so, and the reference harness when `ref_src` (or the
    environment's REF) names the reference checkout."""
    cmd = ["make", "-s", "-C", str(HERE)]
    ref_src = ref_src or os.environ.get("REF")
    if ref_src:
        cmd.append(f"REF={ref_src}")
    subprocess.run(cmd, check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp, i32, f32 = C.c_void_p, C.c_int, C.c_float
        L.vjo_feature_pool.restype = C.c_int64
        L.vjo_feature_pool.argtypes = [i32, i32, i32, vp, C.c_int64]
        L.vjo_integral.argtypes = [vp, i32, i32, i32, vp, vp]
        L.vjo_train_integrals.argtypes = [vp, i32, vp, vp]
        L.vjo_train_response.restype = f32
        L.vjo_train_response.argtypes = [vp, vp, f32]
        L.vjo_weak_search.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, i32, i32, C.POINTER(Best), vp]
        L.vjo_feature_err64.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, i32, i32, vp]
        L.vjo_sorted_build.restype = vp
        L.vjo_sorted_build.argtypes = [vp, i32, vp, vp, i32, i32]
        L.vjo_sorted_search.argtypes = [vp, vp, vp, vp, vp, i32, C.POINTER(Best), vp]
        L.vjo_sorted_free.argtypes = [vp]
        L.vjo_round_update.argtypes = [vp, C.POINTER(Best), vp, vp, vp, vp, vp, vp, i32, vp]
        L.vjo_stage_calibrate.argtypes = [vp, vp, i32, i32, f32, f32, i32, vp, vp]
        L.vjo_resize.argtypes = [vp, i32, i32, i32, vp, i32, i32]
        L.vjo_detect.restype = i32
        L.vjo_detect.argtypes = [vp, i32, vp, i32, vp, i32, i32, i32, vp, i32, i32, i32, f32, i32, i32, i32, i32,
                                 i32, vp, i32]
        L.vjo_group.restype = i32
        L.vjo_group.argtypes = [vp, i32, i32, f32, vp]
        L.vjo_group_first_order.restype = i32
        L.vjo_group_first_order.argtypes = [vp, i32, i32, f32, vp]
        L.vjo_crop_resize.restype = None
        L.vjo_crop_resize.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, i32, vp]
        L.vjo_synth_patches.restype = None
        L.vjo_synth_patches.argtypes = [C.c_uint64, i32, i32, vp]
        L.vjo_synth_scene.restype = i32
        L.vjo_synth_scene.argtypes = [C.c_uint64, i32, i32, i32, i32, i32, vp]
        L.vjo_synth_cascade.restype = i32
        L.vjo_synth_cascade.argtypes = [C.c_uint64, i32, i32, vp, vp]
        _lib = L
    return _lib


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    """The reference's CPU functions (built only where the reference sources are)."""
    global _ref
    if _ref is None:
        R = C.CDLL(str(REF_LIB))
        vp, i32, f32 = C.c_void_p, C.c_int, C.c_float
        R.ref_pool.restype = C.c_longlong
        R.ref_pool.argtypes = [i32, vp, C.c_longlong]
        R.ref_integral.argtypes = [vp, i32, i32, i32, vp, vp, vp]
        R.ref_weak_search.argtypes = [vp, i32, vp, i32, vp, vp, vp, vp, vp, vp, vp]
        R.ref_resize.argtypes = [vp, i32, i32, i32, vp, i32, i32]
        R.ref_crop.argtypes = [vp, i32, i32, i32, i32, i32, i32, vp]
        R.ref_detect.restype = i32
        R.ref_detect.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, i32, i32, f32, i32, i32, i32, vp, i32]
        R.ref_group.restype = i32
        R.ref_group.argtypes = [vp, i32, i32, f32, vp, i32]
        R.ref_model_save.restype = i32
        R.ref_model_save.argtypes = [C.c_char_p, vp, C.c_longlong, vp, C.c_longlong, vp, C.c_longlong]
        _ref = R
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data


def feature_pool(mode: int = 0, win: int = 24) -> np.ndarray:
    n = lib().vjo_feature_pool(mode, win, win, None, 0)
    out = np.zeros(n, dtype=FEATURE)
    lib().vjo_feature_pool(mode, win, win, _p(out), n)
    return out


def integral(img: np.ndarray):
    h, w = img.shape
    img = np.ascontiguousarray(img, dtype=np.uint8)
    s = np.zeros((h + 1, w + 1), dtype=np.uint32)
    q = np.zeros((h + 1, w + 1), dtype=np.uint64)
    lib().vjo_integral(_p(img), w, h, w, _p(s), _p(q))
    return s, q


def train_integrals(patches: np.ndarray):
    patches = np.ascontiguousarray(patches, dtype=np.uint8)
    n = patches.shape[0]
    sums = np.zeros((n, 625), dtype=np.uint32)
    inv = np.zeros(n, dtype=np.float32)
    lib().vjo_train_integrals(_p(patches), n, _p(sums), _p(inv))
    return sums, inv


def weak_search(feats, sums, inv, labels, weights, active=None, used=None, threads=8, per_feature=False):
    b = Best()
    n = len(labels)
    per = np.zeros(len(feats), dtype=BEST) if per_feature else None
    lib().vjo_weak_search(_p(feats), len(feats), _p(used), _p(sums), _p(inv), _p(labels), _p(active),
                          _p(weights), n, threads, C.byref(b), _p(per))
    return (b.as_dict(), per) if per_feature else b.as_dict()


class SortedPool:
    """Stage-resident form of weak_search: every feature of `feats` sorted once
    (6 bytes of host memory per feature-sample), then search() per round with
    the same sweep and pick rule as weak_search."""

    def __init__(self, feats, sums, inv, threads=8):
        self.feats = np.ascontiguousarray(feats)
        self.n = len(inv)
        self.h = lib().vjo_sorted_build(_p(self.feats), len(self.feats), _p(sums), _p(inv), self.n, threads)
        if not self.h:
            raise MemoryError("vjo_sorted_build: out of host memory")

    def search(self, labels, weights, active=None, used=None, threads=8, per_feature=False):
        b = Best()
        per = np.zeros(len(self.feats), dtype=BEST) if per_feature else None
        lib().vjo_sorted_search(self.h, _p(used), _p(labels), _p(active), _p(weights), threads, C.byref(b),
                                _p(per))
        return (b.as_dict(), per) if per_feature else b.as_dict()

    def close(self):
        if self.h:
            lib().vjo_sorted_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def feature_err64(feats, sums, inv, labels, weights, active=None, used=None, threads=8):
    out = np.zeros(len(feats), dtype=np.float64)
    lib().vjo_feature_err64(_p(feats), len(feats), _p(used), _p(sums), _p(inv), _p(labels), _p(active),
                            _p(weights), len(labels), threads, _p(out))
    return out


def round_update(feats, best: dict, sums, inv, labels, weights, strong, active=None):
    """Updates weights and strong in place; returns (theta, err, alpha, left, right, parity, featureIdx)."""
    b = Best(best["featureIdx"], best["err"], best["theta"], best["parity"], best.get("split", -1), 0.0)
    out = np.zeros(7, dtype=np.float32)
    lib().vjo_round_update(_p(feats), C.byref(b), _p(sums), _p(inv), _p(labels), _p(active), _p(weights),
                           _p(strong), len(labels), _p(out))
    return out


def stage_calibrate(strong, num_pos, min_hit, max_fa, neg_base, active=None):
    f = np.zeros(4, dtype=np.float32)
    i = np.zeros(4, dtype=np.int32)
    lib().vjo_stage_calibrate(_p(strong), _p(active), len(strong), num_pos, min_hit, max_fa, neg_base, _p(f), _p(i))
    return dict(cutVal=f[0], stageThreshold=f[1], hitRate=f[2], falseAlarm=f[3], strictGt=int(i[0]),
                posPass=int(i[1]), negSurvive=int(i[2]), satisfied=int(i[3]))


def resize(src: np.ndarray, dw: int, dh: int) -> np.ndarray:
    src = np.ascontiguousarray(src, dtype=np.uint8)
    out = np.zeros((dh, dw), dtype=np.uint8)
    lib().vjo_resize(_p(src), src.shape[1], src.shape[0], src.shape[1], _p(out), dw, dh)
    return out


def detect(feats, stumps, stages, img, sf=1.25, min_obj=24, max_det=200000, max_scales=0, norm_mode=0,
           threads=8, cap=None):
    img = np.ascontiguousarray(img, dtype=np.uint8)
    cap = cap or max_det
    out = np.zeros(cap, dtype=DET)
    n = lib().vjo_detect(_p(feats), len(feats), _p(stumps), len(stumps), _p(stages), len(stages), 24, 24, _p(img),
                         img.shape[1], img.shape[0], img.shape[1], sf, min_obj, max_det, max_scales, norm_mode,
                         threads, _p(out), cap)
    return out[:n].copy()


def group(dets, min_neighbors=4, eps=0.2):
    dets = np.ascontiguousarray(dets, dtype=DET)
    out = np.zeros(max(1, len(dets)), dtype=DET)
    n = lib().vjo_group(_p(dets), len(dets), min_neighbors, eps, _p(out))
    return out[:n].copy()


def group_first_order(dets, min_neighbors=4, eps=0.2):
    """group() with the clusters ordered by their first member's input index."""
    dets = np.ascontiguousarray(dets, dtype=DET)
    out = np.zeros(max(1, len(dets)), dtype=DET)
    n = lib().vjo_group_first_order(_p(dets), len(dets), min_neighbors, eps, _p(out))
    return out[:n].copy()


def crop_resize(img, box, out=24):
    """cropResizeTo24 of box = (x, y, w, h) from a 2-D uint8 image."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    dst = np.zeros((out, out), np.uint8)
    x, y, w, h = (int(v) for v in box)
    lib().vjo_crop_resize(_p(img), img.shape[1], img.shape[0], img.shape[1], x, y, w, h, out, _p(dst))
    return dst


def synth_patches(seed: int, n_pos: int, n_neg: int) -> np.ndarray:
    """n_pos face patterns then n_neg texture patches, (n, 24, 24) uint8."""
    out = np.zeros((n_pos + n_neg, 24, 24), np.uint8)
    lib().vjo_synth_patches(seed, n_pos, n_neg, _p(out))
    return out


def synth_scene(seed: int, w: int, h: int, n_paste: int, min_size: int = 24, max_size: int = 300) -> np.ndarray:
    out = np.zeros((h, w), np.uint8)
    if lib().vjo_synth_scene(seed, w, h, n_paste, min_size, max_size, _p(out)) != 0:
        raise ValueError("synth_scene: bad arguments")
    return out


def synth_cascade(seed: int, stages: int = 38, stumps: int = 6061):
    """(stumps, stages) of the synthetic cascade over the Basic pool."""
    st = np.zeros(stumps, STUMP)
    sg = np.zeros(stages, STAGE)
    if lib().vjo_synth_cascade(seed, stages, stumps, _p(st), _p(sg)) != 0:
        raise ValueError("synth_cascade: bad arguments")
    return st, sg
