"""C ABI: the library loads, exports every declared symbol, and its host-side
logic (pool, model file, grouping, synthetic inputs) works without a GPU."""
import ctypes as C
import hashlib
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(vj_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(vj):
    lib = vj.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares each of them
    from cs677s26_gb300._capi import SIGNATURES
    assert set(names) <= set(SIGNATURES), set(names) - set(SIGNATURES)


def test_struct_layouts_match_reference(vj):
    assert vj.HAAR_FEATURE.itemsize == 64
    assert vj.STUMP4.itemsize == 16
    assert vj.STAGE.itemsize == 12
    assert vj.DETECTION.itemsize == 24
    assert vj.TILE_BEST.itemsize == 16
    assert vj.FEATURE_BEST.itemsize == 16
    assert vj.WEAK.itemsize == 28


def test_build_info(vj):
    assert b"sm_103a" in vj.load().vj_build_info()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_feature_pool_matches_reference(vj, golden, mode):
    pool = vj.feature_pool(mode)
    g = golden["pool"][str(mode)]
    assert len(pool) == g["count"]
    assert hashlib.sha256(pool.tobytes()).hexdigest() == g["sha256"]


def test_pool_counts(vj):
    assert vj.FaceVisionEngine.countHaarFeatures((24, 24), vj.FeatureMode.Basic) == 162336
    assert vj.FaceVisionEngine.countHaarFeatures((24, 24), vj.FeatureMode.Core) == 210400


def test_pool_capacity_error(vj):
    from cs677s26_gb300 import _capi
    n = C.c_int64()
    buf = np.zeros(10, dtype=vj.HAAR_FEATURE)
    st = _capi.status("vj_feature_pool_build", 0, 24, 24, buf.ctypes.data, 10, C.byref(n))
    assert st == 1 and n.value == 162336


def test_model_file_bytes_match_reference(vj, golden, gin, basic_pool, tmp_path):
    st, sg = gin["det_stumps"], gin["det_stages"]
    p = tmp_path / "m.bin"
    assert vj.ModelIO.saveCascadeModel(str(p), (24, 24), basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4),
                                       sg.view(vj.STAGE))
    data = p.read_bytes()
    assert len(data) == golden["model_file"]["bytes"]
    assert hashlib.sha256(data).hexdigest() == golden["model_file"]["sha256"]
    win, f, s, g = vj.ModelIO.loadCascadeModel(str(p))
    assert win == (24, 24) and f.tobytes() == basic_pool.tobytes()
    assert s.tobytes() == st.tobytes() and g.tobytes() == sg.tobytes()


def test_model_file_rejects_bad_input(vj, tmp_path, basic_pool, gin):
    st, sg = gin["det_stumps"], gin["det_stages"]
    good = tmp_path / "g.bin"
    assert vj.ModelIO.saveCascadeModel(str(good), (24, 24), basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4),
                                       sg.view(vj.STAGE))
    raw = good.read_bytes()
    bad_magic = tmp_path / "m1.bin"
    bad_magic.write_bytes(b"VJCBIN2\0" + raw[8:])
    truncated = tmp_path / "m2.bin"
    truncated.write_bytes(raw[:-5])
    empty_stages = tmp_path / "m3.bin"
    empty_stages.write_bytes(raw[:40] + (0).to_bytes(8, "little") + raw[48:])
    bad_version = tmp_path / "m4.bin"
    bad_version.write_bytes(raw[:8] + (2).to_bytes(4, "little") + raw[12:])
    for p in (bad_magic, truncated, empty_stages, bad_version, tmp_path / "missing.bin"):
        assert vj.ModelIO.loadCascadeModel(str(p)) is None
    # saving refuses empty arrays, like the reference
    assert not vj.ModelIO.saveCascadeModel(str(tmp_path / "e.bin"), (24, 24), basic_pool[:0].view(vj.HAAR_FEATURE),
                                           st.view(vj.STUMP4), sg.view(vj.STAGE))


def test_group_rectangles_matches_reference(vj, gin, golden):
    from cs677s26_gb300 import _capi
    for g in golden["detect"]:
        raw = np.ascontiguousarray(gin[f"det_raw_{g['key']}"]).view(vj.DETECTION)
        out = np.zeros(max(1, len(raw)), dtype=vj.DETECTION)
        n = C.c_int()
        _capi.call("vj_group_rectangles", raw.ctypes.data, len(raw), 4, C.c_float(0.2), out.ctypes.data, C.byref(n))
        assert out[: n.value].tobytes() == gin[f"det_grouped_{g['key']}"].tobytes()


def test_group_rectangles_edge_cases(vj, oracle):
    from cs677s26_gb300 import _capi
    rng = np.random.default_rng(3)
    for trial in range(20):
        n = int(rng.integers(0, 300))
        d = np.zeros(n, dtype=vj.DETECTION)
        d["x"] = rng.integers(0, 200, n)
        d["y"] = rng.integers(0, 200, n)
        s = rng.integers(24, 60, n)
        d["w"] = s
        d["h"] = s
        d["scaleIdx"] = rng.integers(0, 5, n)
        d["score"] = rng.integers(0, 4, n).astype(np.float32)  # ties in bestScore
        out = np.zeros(max(1, n), dtype=vj.DETECTION)
        cnt = C.c_int()
        mn = int(rng.integers(0, 6))
        _capi.call("vj_group_rectangles", d.ctypes.data, n, mn, C.c_float(0.2), out.ctypes.data, C.byref(cnt))
        ref = oracle.group(d.view(oracle.DET), mn, 0.2)
        assert out[: cnt.value].tobytes() == ref.tobytes()


def test_synthetic_inputs_are_deterministic(vj, golden):
    p = vj.synth_patches(677, 2000, 2000)
    assert hashlib.sha256(p.tobytes()).hexdigest() == golden["full_pool_round1_4k"]["patches_sha256"]
    a = vj.synth_scene(5, 333, 177, 3, 24, 100)
    b = vj.synth_scene(5, 333, 177, 3, 24, 100)
    assert a.tobytes() == b.tobytes()
    st1, sg1 = vj.synth_cascade(2, 12, 400)
    st2, sg2 = vj.synth_cascade(2, 12, 400)
    assert st1.tobytes() == st2.tobytes() and sg1.tobytes() == sg2.tobytes()
    assert list(sg1["ntrees"][:5]) == [1, 10, 25, 25, 50]


def test_synthetic_cascade_shape(vj):
    st, sg = vj.synth_cascade(7, 38, 6061)
    sizes = list(sg["ntrees"])
    assert sizes[:5] == [1, 10, 25, 25, 50]
    assert sizes[5:15] == [181] * 10 and sizes[15:] == [180] * 23
    assert sum(sizes) == 6061 and sg["first"][-1] + sizes[-1] == 6061
    fi = vj.feature_index(st)
    assert fi.min() >= 0 and fi.max() < 162336


def test_synthetic_statistics(vj):
    p = vj.synth_patches(1, 500, 500)
    neg = p[500:].astype(np.float64)
    assert abs(neg.mean() - 110) < 3 and abs(neg.std() - 45) < 4


def test_invalid_arguments_fail_loudly(vj):
    from cs677s26_gb300 import _capi
    h = C.c_void_p()
    assert _capi.status("vj_trainer_create", 24, 24, 70000, C.byref(h)) == 1
    assert _capi.status("vj_trainer_create", 20, 20, 100, C.byref(h)) == 1
    assert _capi.status("vj_detector_create", 24, 24, 0, 10, 10, C.byref(h)) == 1
    assert b"invalid" in vj.load().vj_last_error()
    with pytest.raises(vj.VJError):
        vj.synth_cascade(1, 0, 10)


def test_detect_estimate_bytes_grows_with_the_image(vj):
    sizes = [(320, 240), (640, 480), (1920, 1080), (3840, 2160)]
    est = [vj.estimate_detect_bytes(w, h) for w, h in sizes]
    assert all(a < b for a, b in zip(est, est[1:]))
    # at least the image, its sums (4 B) and squared sums (8 B) per pixel
    assert est[2] > 1920 * 1080 * 13
    assert vj.estimate_detect_bytes(20, 20) > 0  # smaller than the window: no level, the image copy only


def test_server_config_is_validated(vj, basic_pool):
    """Bad server configurations are refused before any device work."""
    st, sg = vj.synth_cascade(2)
    f, s, g = basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4), sg.view(vj.STAGE)
    for bad in (dict(workers=0), dict(maxBatchImages=0), dict(hbmBudgetBytes=0), dict(scaleFactor=1.0),
                dict(blocksPerSM=-1), dict(maxBatchPixels=-1)):
        with pytest.raises(vj.VJError) as ei:
            vj.DetectServer(f, s, g, **bad)
        assert ei.value.status == vj.Status.kInvalidArg


def test_group_rectangles_large_input_matches_oracle(vj, oracle, basic_pool):
    """Thousands of raw detections from the oracle's detect restatement: the
    library's grouping (swept from x-sorted arrays with a y prefilter) gives
    the oracle's clusters in the oracle's order."""
    st, sg = vj.synth_cascade(2)
    scene = vj.synth_scene(7, 800, 600, 12, 24, 200)
    raw = oracle.detect(basic_pool, st, sg, scene, norm_mode=0, threads=8)
    assert len(raw) > 1000
    lib = vj.load()
    for minn in (1, 4, 8):
        out = np.zeros(len(raw), dtype=vj.DETECTION)
        n = C.c_int()
        assert lib.vj_group_rectangles(raw.ctypes.data, len(raw), minn, C.c_float(0.2), out.ctypes.data,
                                       C.byref(n)) == 0
        assert out[: n.value].tobytes() == oracle.group(raw, minn, 0.2).tobytes()


def test_oracle_first_member_order_is_a_permutation(vj, oracle, basic_pool):
    """The oracle's first-member ordering (the device grouping's output order)
    holds the same clusters as its reference-order grouping."""
    st, sg = vj.synth_cascade(2)
    scene = vj.synth_scene(7, 800, 600, 12, 24, 200)
    raw = oracle.detect(basic_pool, st, sg, scene, norm_mode=0, threads=8)
    for minn in (0, 2, 4):
        a, b = oracle.group(raw, minn, 0.2), oracle.group_first_order(raw, minn, 0.2)
        assert len(a) == len(b) > 0
        assert sorted(x.tobytes() for x in a) == sorted(x.tobytes() for x in b)
