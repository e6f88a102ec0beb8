"""Pins the CPU oracle to the reference: every fixture in tests/golden/ is an
output of the reference's own CPU functions (tests/golden/make_golden.py)."""
import hashlib

import numpy as np
import pytest

from conftest import f32


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_pool(oracle, golden, mode):
    p = oracle.feature_pool(mode)
    assert len(p) == golden["pool"][str(mode)]["count"]
    assert sha(p) == golden["pool"][str(mode)]["sha256"]


def test_integral_images(oracle, golden, gin):
    for g in golden["integral"]:
        img = gin[g["key"]]
        s, q = oracle.integral(img)
        assert sha(s.astype(np.uint32)) == g["sum"]
        assert sha(q.astype(np.uint32)) == g["sqsum"]  # the reference keeps the low 32 bits


def test_integral_wraps_like_reference(oracle, golden):
    g = golden["integral_white"]
    s, q = oracle.integral(np.full((g["h"], g["w"]), 255, np.uint8))
    assert sha(s) == g["sum"] and sha(q.astype(np.uint32)) == g["sqsum"]
    assert q.max() > 2**32  # exact squared sums exceed 32 bits here


def test_train_invnorm(oracle, golden, gin):
    for g in golden["integral"]:
        img = gin[g["key"]]
        if img.shape != (24, 24):
            continue
        _, inv = oracle.train_integrals(img[None])
        assert int(inv.view(np.uint32)[0]) == g["invNorm_bits"]


def test_resize(oracle, golden, gin):
    for g in golden["resize"]:
        assert sha(oracle.resize(gin["resize_src"], g["dw"], g["dh"])) == g["sha256"]


def _case(gin, pool, key):
    idx = gin[key + "_idx"]
    return (np.ascontiguousarray(pool[idx]), gin[key + "_w"], gin.get(key + "_active"))


def test_weak_search_cases(oracle, golden, gin, basic_pool):
    patches = gin["ws_patches"]
    sums, inv = oracle.train_integrals(patches)
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    assert inv[7] == 0.0 and inv[200] == 0.0  # flat patches
    for g in golden["weak_search"]:
        feats, w, act = _case(gin, basic_pool, g["key"])
        b = oracle.weak_search(feats, sums, inv, labels, w, active=act)
        assert b["featureIdx"] == g["featureIdx"], g
        assert b["err"] == f32(g["err_bits"]) and b["theta"] == f32(g["theta_bits"]) and b["parity"] == g["parity"]


def test_rounds_with_fp64_update(oracle, golden, vj, basic_pool):
    g = golden["rounds"]
    p = vj.synth_patches(g["seed"], g["npos"], g["nneg"])
    assert sha(p) == g["patches_sha256"]
    labels = np.array([1] * g["npos"] + [-1] * g["nneg"], np.int8)
    feats = np.ascontiguousarray(basic_pool[: g["features"]])
    sums, inv = oracle.train_integrals(p)
    w = np.full(len(labels), np.float32(0.5) / np.float32(g["npos"]), np.float32)
    strong = np.zeros(len(labels), np.float32)
    used = np.zeros(len(feats), np.uint8)
    for r in g["picks"]:
        b = oracle.weak_search(feats, sums, inv, labels, w, used=used)
        assert (b["featureIdx"], b["err"], b["theta"], b["parity"]) == (
            r["featureIdx"], f32(r["err_bits"]), f32(r["theta_bits"]), r["parity"])
        oracle.round_update(feats, b, sums, inv, labels, w, strong)
        used[b["featureIdx"]] = 1
        assert abs(w.sum(dtype=np.float64) - 1.0) < 1e-5


@pytest.mark.slow
def test_full_pool_round1_4k_full_pool(oracle, golden, vj, basic_pool):
    g = golden["full_pool_round1_4k"]
    p = vj.synth_patches(677, 2000, 2000)
    sums, inv = oracle.train_integrals(p)
    labels = np.array([1] * 2000 + [-1] * 2000, np.int8)
    w = np.full(4000, np.float32(0.5) / np.float32(2000), np.float32)
    b = oracle.weak_search(basic_pool, sums, inv, labels, w, threads=8)
    assert (b["featureIdx"], b["err"], b["theta"], b["parity"]) == (
        g["featureIdx"], f32(g["err_bits"]), f32(g["theta_bits"]), g["parity"])


def test_detect_raw_and_grouped(oracle, golden, gin, basic_pool):
    st, sg = gin["det_stumps"], gin["det_stages"]
    for g in golden["detect"]:
        scene = gin[f"det_scene_{g['key']}"]
        raw = oracle.detect(basic_pool, st, sg, scene, norm_mode=1)
        assert len(raw) == g["raw"]
        assert raw.tobytes() == gin[f"det_raw_{g['key']}"].tobytes()
        grp = oracle.group(raw, 4, 0.2)
        assert grp.tobytes() == gin[f"det_grouped_{g['key']}"].tobytes()


def test_detect_truncation(oracle, golden, gin, basic_pool):
    st, sg = gin["det_stumps"], gin["det_stages"]
    raw = oracle.detect(basic_pool, st, sg, gin["det_scene_0"], max_det=golden["detect_trunc"]["maxDetections"],
                        norm_mode=1)
    assert raw.tobytes() == gin["det_trunc"].tobytes()


def test_detect_norm_modes_agree_below_2_24(oracle, gin, basic_pool):
    # On small scenes no integral value reaches 2^24, so float corners are exact.
    st, sg = gin["det_stumps"], gin["det_stages"]
    scene = gin["det_scene_2"]
    assert np.array_equal(oracle.detect(basic_pool, st, sg, scene, norm_mode=0),
                          oracle.detect(basic_pool, st, sg, scene, norm_mode=1))


def test_stage_calibration_rules(oracle):
    rng = np.random.default_rng(1)
    strong = rng.normal(size=1000).astype(np.float32)
    strong[:10] = strong[5]  # ties at the cut
    c = oracle.stage_calibrate(strong, 500, np.float32(0.99), np.float32(0.4), 500)
    ps = np.sort(strong[:500])
    cut_idx = 500 - int(np.ceil(np.float32(0.99) * np.float32(500)))
    assert c["cutVal"] == ps[cut_idx]
    assert c["posPass"] >= 495 or c["strictGt"] == 0


def test_crop_resize(oracle, golden, gin):
    """cropResizeTo24 (main.cu:245-284): the oracle against the reference's own
    function on border, empty, non-square, oversized and random windows."""
    img, boxes, out = gin["crop_img"], gin["crop_boxes"], gin["crop_out"]
    assert len(boxes) == golden["crop"]["boxes"]
    for k, b in enumerate(boxes):
        assert np.array_equal(oracle.crop_resize(img, b).reshape(-1), out[k]), tuple(b)


def test_tilted_features_like_the_reference(oracle, golden, gin):
    """Tilted (All-mode) features: the reference evaluates their corner indices
    on the upright integral; the oracle's search, detection and grouping over
    them equal the reference's."""
    allp = oracle.feature_pool(2)
    patches = gin["ws_patches"]
    sums, inv = oracle.train_integrals(patches)
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    for g in golden["tilted_weak_search"]:
        feats = np.ascontiguousarray(allp[gin[g["key"] + "_idx"]])
        b = oracle.weak_search(feats, sums, inv, labels, gin[g["key"] + "_w"])
        assert b["featureIdx"] == g["featureIdx"]
        assert b["err"] == f32(g["err_bits"]) and b["theta"] == f32(g["theta_bits"]) and b["parity"] == g["parity"]
    raw = oracle.detect(allp, gin["tdet_stumps"], gin["tdet_stages"], gin["tdet_scene"], threads=8)
    assert len(raw) == golden["tilted_detect"]["raw"] and raw.tobytes() == gin["tdet_raw"].tobytes()
    assert oracle.group(raw, 4, 0.2).tobytes() == gin["tdet_grouped"].tobytes()
