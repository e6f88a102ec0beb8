"""Generates tests/golden/ fixtures from the reference's own CPU functions.

The reference (hengyizhu/CS677s26) ships no tests or golden vectors, so these
are outputs of its CPU paths - buildHaarFeaturePool, buildHostIntegralImage,
runCpuWeakSearch, resizeGrayBilinearHost, detectMultiScaleCpu,
groupRectanglesCpu, cropResizeTo24 and ModelIO::saveCascadeModel (also over tilted
features) - compiled from its sources
by oracle/Makefile into oracle/_ref/libvjref.so (only where the sources are,
i.e. not on the GPU machines).  Inputs are seeded numpy arrays (stored in
inputs.npz) or the package's synthetic generators (their bytes are hashed in
the fixture so a generator change is caught).

    python tests/golden/make_golden.py            # writes golden.json, inputs.npz
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
import cs677s26_gb300 as V  # noqa: E402


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def f32bits(x: float) -> int:
    return int(np.array([x], dtype=np.float32).view(np.uint32)[0])


def ref_search(R, feats, patches, labels, weights, active=None):
    a, e, t, p = C.c_int(), C.c_float(), C.c_float(), C.c_int()
    R.ref_weak_search(feats.ctypes.data, len(feats), patches.ctypes.data, len(labels), labels.ctypes.data,
                      None if active is None else active.ctypes.data, weights.ctypes.data, C.byref(a), C.byref(e),
                      C.byref(t), C.byref(p))
    return dict(featureIdx=a.value, err_bits=f32bits(e.value), theta_bits=f32bits(t.value), parity=p.value)


def main() -> None:
    if not O.ref_available():
        O.build()
    R = O.ref()
    rng = np.random.default_rng(677)
    gold: dict = {"about": "outputs of the reference's CPU functions (see make_golden.py)"}
    inputs: dict = {}

    # ---- feature pools
    gold["pool"] = {}
    for mode in (0, 1, 2):
        n = R.ref_pool(mode, None, 0)
        buf = np.zeros(n, dtype=O.FEATURE)
        R.ref_pool(mode, buf.ctypes.data, n)
        gold["pool"][str(mode)] = {"count": int(n), "sha256": sha(buf)}

    # ---- integral images (int32 sum / sqsum bits) and invNorm
    gold["integral"] = []
    for k, (h, w) in enumerate([(1, 1), (1, 9), (24, 24), (19, 37), (97, 131), (480, 640)]):
        img = rng.integers(0, 256, (h, w), dtype=np.uint8)
        if k == 2:
            img[:] = 200  # flat patch: invNorm 0
        inputs[f"ii_{k}"] = img
        s = np.zeros((h + 1) * (w + 1), np.int32)
        q = np.zeros_like(s)
        inv = np.zeros(1, np.float32)
        R.ref_integral(img.ctypes.data, w, h, w, s.ctypes.data, q.ctypes.data, inv.ctypes.data)
        gold["integral"].append({"key": f"ii_{k}", "sum": sha(s), "sqsum": sha(q), "invNorm_bits": f32bits(inv[0])})
    # a large white image: sums above 2^24 and squared sums wrapping mod 2^32
    big = np.full((300, 400), 255, np.uint8)
    s = np.zeros(301 * 401, np.int32)
    q = np.zeros_like(s)
    inv = np.zeros(1, np.float32)
    R.ref_integral(big.ctypes.data, 400, 300, 400, s.ctypes.data, q.ctypes.data, inv.ctypes.data)
    gold["integral_white"] = {"h": 300, "w": 400, "sum": sha(s), "sqsum": sha(q)}

    # ---- resize
    gold["resize"] = []
    src = rng.integers(0, 256, (101, 173), dtype=np.uint8)
    inputs["resize_src"] = src
    for dw, dh in [(138, 81), (110, 64), (24, 24), (173, 101), (57, 33)]:
        out = np.zeros((dh, dw), np.uint8)
        R.ref_resize(src.ctypes.data, 173, 101, 173, out.ctypes.data, dw, dh)
        gold["resize"].append({"dw": dw, "dh": dh, "sha256": sha(out)})

    # ---- best-weak search on small cases
    pool = O.feature_pool(0)
    patches = V.synth_patches(31, 160, 160)
    patches[7] = 90  # flat positive (invNorm 0 -> -0.0 responses)
    patches[200] = 30  # flat negative
    inputs["ws_patches"] = patches
    n = len(patches)
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    gold["weak_search"] = []
    cases = []
    for c in range(8):
        F = 6000
        idx = np.sort(rng.choice(len(pool), F, replace=False)) if c % 2 else np.arange(F)
        kind = ["uniform", "random", "uniform-inactive", "random-inactive", "ties", "random", "skewed", "random"][c]
        if kind.startswith("uniform") or kind == "ties":
            w = np.full(n, np.float32(0.5) / np.float32(160), np.float32)
        elif kind == "skewed":
            w = (rng.random(n) ** 6).astype(np.float32)
            w /= w.sum(dtype=np.float64)
            w = w.astype(np.float32)
        else:
            w = (rng.random(n) / n).astype(np.float32)
        if kind == "ties":
            w[:] = np.float32(1.0 / 512)  # exactly representable: many exact ties
        act = (rng.random(n) > 0.25).astype(np.uint8) if "inactive" in kind else None
        feats = np.ascontiguousarray(pool[idx])
        r = ref_search(R, feats, patches, labels, w, act)
        key = f"ws_{c}"
        inputs[key + "_idx"] = idx.astype(np.int32)
        inputs[key + "_w"] = w
        if act is not None:
            inputs[key + "_active"] = act
        gold["weak_search"].append({"key": key, "kind": kind, **r})
        cases.append(key)

    # ---- several rounds: weights from the FP64 round update, each round's
    # pick by the reference search over the features not yet used
    mp = V.synth_patches(47, 300, 300)
    ml = np.array([1] * 300 + [-1] * 300, np.int8)
    mF = 20000
    mfeats = np.ascontiguousarray(pool[:mF])
    sums, inv = O.train_integrals(mp)
    w = np.where(ml > 0, np.float32(0.5) / np.float32(300), np.float32(0.5) / np.float32(300)).astype(np.float32)
    strong = np.zeros(len(ml), np.float32)
    used = np.zeros(mF, np.uint8)
    rounds = []
    for r_ in range(6):
        keep = np.nonzero(used == 0)[0]
        r = ref_search(R, np.ascontiguousarray(mfeats[keep]), mp, ml, w)
        r["featureIdx"] = int(keep[r["featureIdx"]])
        rounds.append(r)
        best = dict(featureIdx=r["featureIdx"], err=float(np.uint32(r["err_bits"]).view(np.float32)),
                    theta=float(np.uint32(r["theta_bits"]).view(np.float32)), parity=r["parity"])
        O.round_update(mfeats, best, sums, inv, ml, w, strong)
        used[r["featureIdx"]] = 1
    gold["rounds"] = {"seed": 47, "npos": 300, "nneg": 300, "features": mF, "picks": rounds,
                      "patches_sha256": sha(mp)}

    # ---- 2,000 + 2,000 patches: round 1 over the full Basic pool
    t0 = time.time()
    p0 = V.synth_patches(677, 2000, 2000)
    l0 = np.array([1] * 2000 + [-1] * 2000, np.int8)
    w0 = np.full(4000, np.float32(0.5) / np.float32(2000), np.float32)
    r0 = ref_search(R, np.ascontiguousarray(pool), p0, l0, w0)
    gold["full_pool_round1_4k"] = {"patches_sha256": sha(p0), "seconds": round(time.time() - t0, 1), **r0}

    # ---- detection (raw, scan order) and grouping, small cascade
    st, sg = V.synth_cascade(2, 12, 400)
    gold["detect"] = []
    for k, (w_, h_, npaste) in enumerate([(320, 240, 6), (256, 200, 4), (97, 61, 1)]):
        scene = V.synth_scene(100 + k, w_, h_, npaste, 24, min(w_, h_))
        inputs[f"det_scene_{k}"] = scene
        cap = 200000
        out = np.zeros(cap, O.DET)
        nd = R.ref_detect(pool.ctypes.data, len(pool), st.ctypes.data, len(st), sg.ctypes.data, len(sg),
                          scene.ctypes.data, w_, h_, w_, 1.25, 24, cap, 0, out.ctypes.data, cap)
        raw = out[:nd].copy()
        g = np.zeros(max(1, nd), O.DET)
        ng = R.ref_group(raw.ctypes.data, nd, 4, 0.2, g.ctypes.data, max(1, nd))
        inputs[f"det_raw_{k}"] = raw
        inputs[f"det_grouped_{k}"] = g[:ng].copy()
        gold["detect"].append({"key": k, "w": w_, "h": h_, "raw": int(nd), "grouped": int(ng)})
    inputs["det_stumps"] = st
    inputs["det_stages"] = sg
    # maxDetections truncation and maxScales
    scene = inputs["det_scene_0"]
    out = np.zeros(50, O.DET)
    nd = R.ref_detect(pool.ctypes.data, len(pool), st.ctypes.data, len(st), sg.ctypes.data, len(sg),
                      scene.ctypes.data, 320, 240, 320, 1.25, 24, 50, 0, out.ctypes.data, 50)
    inputs["det_trunc"] = out[:nd].copy()
    gold["detect_trunc"] = {"maxDetections": 50, "raw": int(nd)}

    # ---- cropResizeTo24 of hard-negative windows (main.cu:245-284)
    img = V.synth_scene(300, 203, 151, 2, 24, 100)
    boxes = [(0, 0, 24, 24), (10, 5, 48, 48), (150, 100, 50, 50), (202, 150, 1, 1), (5, 7, 0, 0),
             (37, 11, 31, 17), (-3, -2, 30, 30), (0, 0, 203, 151), (120, 80, 90, 90), (3, 4, 25, 26),
             (60, 40, 23, 23), (100, 30, 300, 7)]
    boxes += [(int(rng.integers(-20, 210)), int(rng.integers(-20, 160)), int(rng.integers(0, 240)),
               int(rng.integers(0, 180))) for _ in range(52)]
    crops = np.zeros((len(boxes), 576), np.uint8)
    for k, (x, y, bw, bh) in enumerate(boxes):
        R.ref_crop(img.ctypes.data, 203, 151, x, y, bw, bh, crops[k].ctypes.data)
    inputs["crop_img"] = img
    inputs["crop_boxes"] = np.array(boxes, np.int32)
    inputs["crop_out"] = crops
    gold["crop"] = {"boxes": len(boxes), "out_sha256": sha(crops)}

    # ---- tilted (All-mode) features: the reference evaluates their four corner
    # indices on the upright integral like any other feature (it never builds a
    # tilted integral); a weak search over them and a cascade that uses them
    trng = np.random.default_rng(1677)
    allp = O.feature_pool(2)
    tidx = np.nonzero(allp["tilted"] == 1)[0]
    gold["tilted_weak_search"] = []
    for c, kind in enumerate(["uniform", "random"]):
        idx = np.sort(trng.choice(tidx, 6000, replace=False))
        w = (np.full(n, np.float32(0.5) / np.float32(160), np.float32) if kind == "uniform"
             else (trng.random(n) / n).astype(np.float32))
        r = ref_search(R, np.ascontiguousarray(allp[idx]), inputs["ws_patches"], labels, w)
        key = f"tws_{c}"
        inputs[key + "_idx"] = idx.astype(np.int32)
        inputs[key + "_w"] = w
        gold["tilted_weak_search"].append({"key": key, "kind": kind, **r})
    # 3 stages x 10 tilted stumps, each stage threshold at the median stage sum
    # of the windows that reach it (from the reference's own detection scores)
    tst = np.zeros(30, dtype=V.STUMP4)
    tst["featureBits"] = trng.choice(tidx, 30).astype(np.int32).view(np.float32)
    tst["theta"] = trng.normal(0, 0.02, 30).astype(np.float32)
    tst["leftVal"], tst["rightVal"] = -1.0, 1.0
    tsg = np.zeros(3, dtype=V.STAGE)
    tscene = V.synth_scene(150, 200, 150, 3, 24, 150)
    cap = 200000
    out = np.zeros(cap, O.DET)
    for k in range(3):
        tsg[k] = (10 * k, 10, np.float32(-1e30))
        nd = R.ref_detect(allp.ctypes.data, len(allp), tst.ctypes.data, len(tst), tsg.ctypes.data, k + 1,
                          tscene.ctypes.data, 200, 150, 200, 1.25, 24, cap, 0, out.ctypes.data, cap)
        tsg[k]["threshold"] = np.float32(np.median(out[:nd]["score"]))
    nd = R.ref_detect(allp.ctypes.data, len(allp), tst.ctypes.data, len(tst), tsg.ctypes.data, 3,
                      tscene.ctypes.data, 200, 150, 200, 1.25, 24, cap, 0, out.ctypes.data, cap)
    traw = out[:nd].copy()
    g = np.zeros(max(1, nd), O.DET)
    ng = R.ref_group(traw.ctypes.data, nd, 4, 0.2, g.ctypes.data, max(1, nd))
    inputs.update(tdet_scene=tscene, tdet_stumps=tst, tdet_stages=tsg, tdet_raw=traw, tdet_grouped=g[:ng].copy())
    gold["tilted_detect"] = {"raw": int(nd), "grouped": int(ng)}

    # ---- model file bytes
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "m.bin"
        R.ref_model_save(str(path).encode(), pool.ctypes.data, len(pool), st.ctypes.data, len(st),
                         sg.ctypes.data, len(sg))
        gold["model_file"] = {"sha256": hashlib.sha256(path.read_bytes()).hexdigest(),
                              "bytes": path.stat().st_size}

    (HERE / "golden.json").write_text(json.dumps(gold, indent=1) + "\n")
    np.savez_compressed(HERE / "inputs.npz", **inputs)
    print(f"wrote {HERE / 'golden.json'} and inputs.npz")


if __name__ == "__main__":
    main()
