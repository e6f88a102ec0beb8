"""GPU parity: the CUDA path, called through the C ABI, against the oracle and
the reference's golden outputs.  Integer work is compared bit for bit; stump
picks (feature, threshold, parity, FP32 error) too."""
import ctypes as C

import numpy as np
import pytest

from conftest import f32

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# ---------------------------------------------------------------- integrals
def test_integral_batch_24(cuda, vj, oracle):
    torch = cuda
    p = vj.synth_patches(9, 300, 300)
    p[3] = 17
    p[400] = 255
    d = dev(torch, p)
    n = len(p)
    sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
    sqT = torch.empty(625 * n, dtype=torch.int64, device="cuda")
    inv = torch.empty(n, dtype=torch.float32, device="cuda")
    vj._capi.call("vj_integral_batch", d.data_ptr(), 24, 24, 24, n, sumT.data_ptr(), sqT.data_ptr(), inv.data_ptr(), None)
    torch.cuda.synchronize()
    sums, oinv = oracle.train_integrals(p)
    assert np.array_equal(sumT.cpu().numpy().view(np.uint32).reshape(625, n).T, sums)
    assert np.array_equal(inv.cpu().numpy().view(np.uint32), oinv.view(np.uint32))
    for i in (0, 3, 400):
        _, q = oracle.integral(p[i])
        assert np.array_equal(sqT.cpu().numpy().view(np.uint64).reshape(625, n)[:, i], q.ravel())


@pytest.mark.parametrize("h,w", [(7, 5), (31, 40)])
def test_integral_batch_generic(cuda, vj, oracle, h, w):
    torch = cuda
    rng = np.random.default_rng(h * w)
    n = 77
    imgs = rng.integers(0, 256, (n, h, w), dtype=np.uint8)
    d = dev(torch, imgs)
    area = (h + 1) * (w + 1)
    sumT = torch.empty(area * n, dtype=torch.int32, device="cuda")
    sqT = torch.empty(area * n, dtype=torch.int64, device="cuda")
    inv = torch.empty(n, dtype=torch.float32, device="cuda")
    vj._capi.call("vj_integral_batch", d.data_ptr(), w, h, w, n, sumT.data_ptr(), sqT.data_ptr(), inv.data_ptr(), None)
    S = sumT.cpu().numpy().view(np.uint32).reshape(area, n)
    Q = sqT.cpu().numpy().view(np.uint64).reshape(area, n)
    for i in (0, 41, 76):
        s, q = oracle.integral(imgs[i])
        assert np.array_equal(S[:, i], s.ravel()) and np.array_equal(Q[:, i], q.ravel())


@pytest.mark.parametrize("h,w", [(1, 1), (24, 24), (61, 97), (300, 400), (480, 640), (1080, 1920), (2160, 3840)])
def test_integral_image(cuda, vj, oracle, h, w):
    torch = cuda
    img = vj.synth_scene(h * 7 + w, w, h, 0) if min(h, w) >= 24 else np.full((h, w), 255, np.uint8)
    if (h, w) == (300, 400):
        img[:] = 255  # sums beyond 2^24, squared sums beyond 2^32
    d = dev(torch, img)
    s = torch.empty((h + 1) * (w + 1), dtype=torch.int32, device="cuda")
    q = torch.empty((h + 1) * (w + 1), dtype=torch.int64, device="cuda")
    vj._capi.call("vj_integral_image", d.data_ptr(), w, h, w, s.data_ptr(), q.data_ptr(), None)
    os_, oq = oracle.integral(img)
    assert np.array_equal(s.cpu().numpy().view(np.uint32), os_.ravel())
    assert np.array_equal(q.cpu().numpy().view(np.uint64), oq.ravel())


# ---------------------------------------------------------------- stump search
class Train:
    """A bound trainer over patches (positives first) with device buffers."""

    def __init__(self, torch, vj, oracle, patches, labels, feats, weights, active=None):
        self.torch, self.vj = torch, vj
        n = len(labels)
        self.n = n
        self.d_p = dev(torch, patches)
        self.sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
        self.inv = torch.empty(n, dtype=torch.float32, device="cuda")
        vj._capi.call("vj_integral_batch", self.d_p.data_ptr(), 24, 24, 24, n, self.sumT.data_ptr(), None,
                      self.inv.data_ptr(), None)
        self.lab = dev(torch, labels.astype(np.int8))
        self.act = dev(torch, active) if active is not None else None
        self.w = dev(torch, weights.astype(np.float32))
        self.t = vj.AdaBoostTrainer((24, 24), n)
        assert self.t.setFeaturePool(feats.view(vj.HAAR_FEATURE)) == 0
        ii = dict(nSamples=n, d_sumT=self.sumT, d_invNorm=self.inv)
        assert self.t.bindTrainingSet(ii, self.lab, self.act, self.w) == 0
        self.best = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.used = torch.zeros(len(feats), dtype=torch.uint8, device="cuda")
        self.strong = torch.zeros(n, dtype=torch.float32, device="cuda")

    def search(self, used=False):
        assert self.t.bestWeak(self.used if used else None, self.best) == 0
        b = self.best.cpu().numpy().view(self.vj.TILE_BEST)[0]
        return int(b["featureIdx"]), float(b["bestErr"]), float(b["bestTheta"]), int(b["bestParity"])


def test_weak_search_golden_cases(cuda, vj, oracle, golden, gin, basic_pool):
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    for g in golden["weak_search"]:
        idx = gin[g["key"] + "_idx"]
        T = Train(cuda, vj, oracle, patches, labels, np.ascontiguousarray(basic_pool[idx]), gin[g["key"] + "_w"],
                  gin.get(g["key"] + "_active"))
        got = T.search()
        assert got == (g["featureIdx"], f32(g["err_bits"]), f32(g["theta_bits"]), g["parity"]), g


def test_weak_search_resident_equals_fused(cuda, vj, oracle, gin, basic_pool):
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    rng = np.random.default_rng(4)
    w = (rng.random(320) / 320).astype(np.float32)
    T = Train(cuda, vj, oracle, patches, labels, np.ascontiguousarray(basic_pool[:20000]), w)
    fused = T.search()
    assert T.t.prepareStage() == 0
    assert T.search() == fused


@pytest.mark.parametrize("n", [16385, 20000, 20480, 24576, 25600, 32768])
def test_weak_search_both_weight_layouts(cuda, vj, oracle, basic_pool, n):
    """Up to 24,576 samples the resident orders carry slots of two bank-spread
    weight copies; above that one copy and plain sample indices, up to the
    on-chip sort's maximum of 32,768.  From 16,385 to 20,480 samples the sort
    is the blocked form with per-thread digit counters.  All give the oracle's
    pick, round after round."""
    p = vj.synth_patches(31, n // 2, n // 2)
    labels = np.array([1] * (n // 2) + [-1] * (n // 2), np.int8)
    feats = np.ascontiguousarray(basic_pool[::317][:512])
    rng = np.random.default_rng(n)
    w = (rng.random(n) / n).astype(np.float32)
    T = Train(cuda, vj, oracle, p, labels, feats, w)
    assert T.t.prepareStage() == 0
    sums, inv = oracle.train_integrals(p)
    used = np.zeros(len(feats), np.uint8)
    strong = np.zeros(n, np.float32)
    weak = cuda.zeros(7, dtype=cuda.int32, device="cuda")
    for _ in range(3):
        got = T.search(used=True)
        ref = oracle.weak_search(feats, sums, inv, labels, T.w.cpu().numpy(), used=used, threads=16)
        assert got == (ref["featureIdx"], ref["err"], ref["theta"], ref["parity"])
        assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
        used[got[0]] = 1


@pytest.mark.parametrize("n,with_active", [(32769, False), (40000, False), (65535, False), (40000, True)])
def test_weak_search_beyond_on_chip_sort(cuda, vj, oracle, basic_pool, n, with_active):
    """From 32,769 samples up to the reference's limit of 65,535 (16-bit sample
    indices, boosting_core.cu:704 and :851) the sort keeps its keys and
    indices in a global scratch and the sweep reads one weight copy (from
    shared memory up to 49,152 samples, from global memory above).  The first
    round re-sorts inside the search, the next two use the resident orders;
    every round gives the oracle's pick."""
    npos = n // 2
    p = vj.synth_patches(61, npos, n - npos)
    labels = np.array([1] * npos + [-1] * (n - npos), np.int8)
    feats = np.ascontiguousarray(basic_pool[::317][:512])
    rng = np.random.default_rng(n)
    w = (rng.random(n) / n).astype(np.float32)
    active = (rng.random(n) > 0.2).astype(np.uint8) if with_active else None
    T = Train(cuda, vj, oracle, p, labels, feats, w, active)
    sums, inv = oracle.train_integrals(p)
    used = np.zeros(len(feats), np.uint8)
    weak = cuda.zeros(7, dtype=cuda.int32, device="cuda")
    for r in range(3):
        if r == 1:
            assert T.t.prepareStage() == 0
        got = T.search(used=True)
        ref = oracle.weak_search(feats, sums, inv, labels, T.w.cpu().numpy(), active=active, used=used, threads=16)
        assert got == (ref["featureIdx"], ref["err"], ref["theta"], ref["parity"]), r
        assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
        used[got[0]] = 1


@pytest.mark.parametrize("n", [16385, 18001, 20480, 40001])
def test_step_api_sort_beyond_on_chip_sort(cuda, vj, oracle, basic_pool, n):
    """sortSamplesPerFeature at 16,385 to 20,480 samples (the blocked sort with
    per-thread digit counters) and at 40,001 (keys and indices in a global
    scratch): the stable order of the radix keys, -0.0 before +0.0 (a flat
    patch has invNorm 0)."""
    torch = cuda
    F = 40
    npos = n // 2
    p = vj.synth_patches(63, npos, n - npos)
    p[11] = 77  # flat: responses +-0.0
    labels = np.array([1] * npos + [-1] * (n - npos), np.int8)
    feats = np.ascontiguousarray(basic_pool[::4001][:F])
    T = Train(cuda, vj, oracle, p, labels, feats, np.full(n, np.float32(1.0 / n), np.float32))
    resp = torch.empty(F * n, dtype=torch.float32, device="cuda")
    assert T.t.evaluateFeatureResponses(0, F, resp) == 0
    order = torch.empty(F * n, dtype=torch.int16, device="cuda")
    assert T.t.sortSamplesPerFeature(resp, F, order) == 0
    R = resp.cpu().numpy().reshape(F, n)
    O_ = order.cpu().numpy().view(np.uint16).reshape(F, n)
    bits = R.view(np.uint32)
    keys = np.where(bits >> 31, ~bits, bits | np.uint32(0x80000000))
    for f in range(F):
        assert np.array_equal(O_[f], np.lexsort((np.arange(n), keys[f]))), f


@pytest.mark.parametrize("n", [2, 3, 17, 33, 100, 511, 513, 1000])
def test_weak_search_small_and_ragged_counts(cuda, vj, oracle, basic_pool, n):
    """Sample counts around the sweep's 16-position lane runs, its 512-position
    chunks and the 32-member copy-assignment groups: the oracle's pick, two
    rounds in a row, with the resident orders."""
    npos = max(1, n // 2)
    p = vj.synth_patches(40 + n, npos, n - npos)
    labels = np.array([1] * npos + [-1] * (n - npos), np.int8)
    feats = np.ascontiguousarray(basic_pool[::53][:3000])
    rng = np.random.default_rng(n)
    w = (rng.random(n) / n).astype(np.float32)
    T = Train(cuda, vj, oracle, p, labels, feats, w)
    assert T.t.prepareStage() == 0
    sums, inv = oracle.train_integrals(p)
    used = np.zeros(len(feats), np.uint8)
    weak = cuda.zeros(7, dtype=cuda.int32, device="cuda")
    for _ in range(2):
        got = T.search(used=True)
        ref = oracle.weak_search(feats, sums, inv, labels, T.w.cpu().numpy(), used=used, threads=8)
        assert got == (ref["featureIdx"], ref["err"], ref["theta"], ref["parity"])
        if got[0] < 0:
            break
        assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
        used[got[0]] = 1


def test_weak_search_without_valid_split(cuda, vj, oracle, basic_pool):
    """Identical patches give every feature a single value: no valid split
    anywhere, reported as featureIdx -1 with an infinite error, as the oracle
    does."""
    one = vj.synth_patches(5, 1, 0)
    p = np.ascontiguousarray(np.repeat(one, 40, axis=0))
    labels = np.array([1] * 20 + [-1] * 20, np.int8)
    feats = np.ascontiguousarray(basic_pool[:2000])
    w = np.full(40, np.float32(1.0 / 40), np.float32)
    T = Train(cuda, vj, oracle, p, labels, feats, w)
    sums, inv = oracle.train_integrals(p)
    ref = oracle.weak_search(feats, sums, inv, labels, w)
    assert ref["featureIdx"] == -1
    got = T.search()
    assert got[0] == -1 and got[1] == float("inf") and got[3] == ref["parity"]
    assert T.t.prepareStage() == 0
    assert T.search() == got


def test_rounds_match_reference_and_oracle(cuda, vj, oracle, golden, basic_pool):
    g = golden["rounds"]
    p = vj.synth_patches(g["seed"], g["npos"], g["nneg"])
    labels = np.array([1] * g["npos"] + [-1] * g["nneg"], np.int8)
    feats = np.ascontiguousarray(basic_pool[: g["features"]])
    w0 = np.full(len(labels), np.float32(0.5) / np.float32(g["npos"]), np.float32)
    T = Train(cuda, vj, oracle, p, labels, feats, w0)
    assert T.t.prepareStage() == 0
    sums, inv = oracle.train_integrals(p)
    w = w0.copy()
    strong = np.zeros(len(labels), np.float32)
    weak = cuda.zeros(7, dtype=cuda.int32, device="cuda")
    for r in g["picks"]:
        got = T.search(used=True)
        assert got == (r["featureIdx"], f32(r["err_bits"]), f32(r["theta_bits"]), r["parity"])
        assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
        oracle.round_update(feats, dict(featureIdx=got[0], err=got[1], theta=got[2], parity=got[3]), sums, inv,
                            labels, w, strong)
        gw = T.w.cpu().numpy()
        assert np.max(np.abs(gw.view(np.int32).astype(np.int64) - w.view(np.int32).astype(np.int64))) <= 1
        assert np.array_equal(T.strong.cpu().numpy(), strong)
        wk = weak.cpu().numpy().view(vj.WEAK)[0]
        assert wk["featureIdx"] == got[0] and wk["parity"] == got[3]
        assert wk["leftVal"] == -wk["rightVal"] and (wk["leftVal"] < 0) == (got[3] > 0)
        w = gw.copy()  # continue from the device weights


@pytest.mark.slow
def test_full_pool_round1_4k_full_pool(cuda, vj, oracle, golden, basic_pool):
    g = golden["full_pool_round1_4k"]
    p = vj.synth_patches(677, 2000, 2000)
    labels = np.array([1] * 2000 + [-1] * 2000, np.int8)
    w = np.full(4000, np.float32(0.5) / np.float32(2000), np.float32)
    T = Train(cuda, vj, oracle, p, labels, basic_pool, w)
    want = (g["featureIdx"], f32(g["err_bits"]), f32(g["theta_bits"]), g["parity"])
    assert T.search() == want
    assert T.t.prepareStage() == 0
    assert T.search() == want


def test_step_api_matches_oracle(cuda, vj, oracle, gin, basic_pool):
    torch = cuda
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    rng = np.random.default_rng(8)
    w = (rng.random(320) / 320).astype(np.float32)
    F = 3000
    feats = np.ascontiguousarray(basic_pool[:F])
    T = Train(cuda, vj, oracle, patches, labels, feats, w)
    n = 320
    resp = torch.empty(F * n, dtype=torch.float32, device="cuda")
    assert T.t.evaluateFeatureResponses(0, F, resp) == 0
    sums, inv = oracle.train_integrals(patches)
    R = resp.cpu().numpy().reshape(F, n)
    for f in (0, 17, 2999):
        ref = np.array([oracle.lib().vjo_train_response(feats[f:f + 1].ctypes.data, sums[i].ctypes.data, inv[i])
                        for i in range(n)], np.float32)
        assert np.array_equal(R[f].view(np.uint32), ref.view(np.uint32))
    order = torch.empty(F * n, dtype=torch.int16, device="cuda")
    assert T.t.sortSamplesPerFeature(resp, F, order) == 0
    O_ = order.cpu().numpy().view(np.uint16).reshape(F, n)
    bits = R.view(np.uint32)
    keys = np.where(bits >> 31, ~bits, bits | np.uint32(0x80000000))
    for f in range(0, F, 97):
        assert np.array_equal(O_[f], np.lexsort((np.arange(n), keys[f])))
    best = torch.empty(F * 4, dtype=torch.int32, device="cuda")
    assert T.t.evaluateAndFindThreshold(resp, order, F, best) == 0
    B = best.cpu().numpy().view(vj.FEATURE_BEST)
    e64 = oracle.feature_err64(feats, sums, inv, labels, w)
    assert np.allclose(B["bestErr"], e64, rtol=0, atol=1e-6)
    tile = torch.zeros(4, dtype=torch.int32, device="cuda")
    assert T.t.selectBestInTile(best, 0, F, None, tile) == 0
    tb = tile.cpu().numpy().view(vj.TILE_BEST)[0]
    assert tb["bestErr"] == B["bestErr"].min() and tb["featureIdx"] == int(np.argmin(B["bestErr"]))


def test_stage_calibration(cuda, vj, oracle, gin, basic_pool):
    torch = cuda
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    T = Train(cuda, vj, oracle, patches, labels, np.ascontiguousarray(basic_pool[:100]),
              np.full(320, np.float32(1 / 320), np.float32))
    rng = np.random.default_rng(2)
    for trial in range(5):
        strong = rng.normal(size=320).astype(np.float32)
        if trial == 1:
            strong[:40] = strong[3]
        if trial == 2:
            strong[:] = np.round(strong * 2) / 2
        d_s = dev(torch, strong)
        out = torch.zeros(8, dtype=torch.int32, device="cuda")
        assert T.t.calibrateStage(d_s, 160, 0.99, 0.4, 160, out) == 0
        got = out.cpu().numpy().view(vj.STAGE_CALIB)[0]
        ref = oracle.stage_calibrate(strong, 160, np.float32(0.99), np.float32(0.4), 160)
        for k in ("cutVal", "stageThreshold", "hitRate", "falseAlarm"):
            assert np.float32(got[k]).tobytes() == np.float32(ref[k]).tobytes(), k
        for k in ("strictGt", "posPass", "negSurvive", "satisfied"):
            assert int(got[k]) == ref[k], k


# ---------------------------------------------------------------- detection
def detector(vj, pool, st, sg, w=3840, h=2160, norm=0):
    e = vj.FaceVisionEngine((24, 24), 1, w, h, False, 200000)
    assert e.setCascadeModel(pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4), sg.view(vj.STAGE)) == 0
    assert e.setNormMode(norm) == 0
    return e


def as_set(dets):
    """Detections as a sorted list of records (groupRectangles' output order
    is not part of the reference's contract)."""
    return sorted(bytes(r) for r in np.ascontiguousarray(dets).view(np.uint8).reshape(-1, 24))


def test_detect_golden(cuda, vj, oracle, golden, gin, basic_pool):
    e = detector(vj, basic_pool, gin["det_stumps"], gin["det_stages"], norm=1)
    for g in golden["detect"]:
        scene = gin[f"det_scene_{g['key']}"]
        st, raw = e.detectMultiScale(scene, g["w"], g["h"], g["w"], 1.25, 4, 24, 200000, applyGrouping=False)
        assert st == 0 and raw.tobytes() == gin[f"det_raw_{g['key']}"].tobytes()
        st, grp = e.detectMultiScale(scene, g["w"], g["h"], g["w"], 1.25, 4, 24, 200000, applyGrouping=True)
        # grouped on the device: the reference's clusters, in first-member order
        assert st == 0 and as_set(grp) == as_set(gin[f"det_grouped_{g['key']}"])
        assert grp.tobytes() == oracle.group_first_order(raw, 4, 0.2).tobytes()
    st, raw = e.detectMultiScale(gin["det_scene_0"], 320, 240, 320, 1.25, 4, 24, 50, applyGrouping=False)
    assert raw.tobytes() == gin["det_trunc"].tobytes()


@pytest.mark.parametrize("norm", [0, 1])
def test_detect_1080p_full_cascade(cuda, vj, oracle, basic_pool, norm):
    st, sg = vj.synth_cascade(2)
    scene = vj.synth_scene(1, 1920, 1080, 40, 24, 300)
    e = detector(vj, basic_pool, st, sg, norm=norm)
    s, raw = e.detectMultiScale(scene, 1920, 1080, 1920, 1.25, 4, 24, 200000, applyGrouping=False)
    ref = oracle.detect(basic_pool, st, sg, scene, norm_mode=norm, threads=8)
    assert s == 0 and len(raw) == len(ref) and raw.tobytes() == ref.tobytes()
    s, grp = e.detectMultiScale(scene, 1920, 1080, 1920, 1.25, 4, 24, 200000)
    assert s == 0 and grp.tobytes() == oracle.group_first_order(ref, 4, 0.2).tobytes()
    assert as_set(grp) == as_set(oracle.group(ref, 4, 0.2))


def test_device_grouping_parameters_and_batches(cuda, vj, oracle, basic_pool):
    """Device groupRectangles against the oracle's restatement of
    groupRectanglesCpu over the canonical raw list: every minNeighbors branch
    (the containment test's n < 3 case included), truncation to
    maxDetections before grouping, and a batch grouped image by image."""
    st, sg = vj.synth_cascade(2)
    e = detector(vj, basic_pool, st, sg)
    scenes = [vj.synth_scene(1, 1920, 1080, 40, 24, 300), vj.synth_scene(7, 800, 600, 12, 24, 200),
              vj.synth_scene(9, 333, 251, 3, 24, 120)]
    raws = []
    for sc in scenes:
        h, w = sc.shape
        s, raw = e.detectMultiScale(sc, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
        assert s == 0
        raws.append(raw)
    assert len(raws[0]) > 5000  # dense clusters around the pasted faces
    for mn in (0, 1, 2, 3, 6):
        for sc, raw in zip(scenes, raws):
            h, w = sc.shape
            s, grp = e.detectMultiScale(sc, w, h, w, 1.25, mn, 24, 200000)
            assert s == 0 and grp.tobytes() == oracle.group_first_order(raw, mn, 0.2).tobytes(), (mn, w)
    for lim in (1, 37, 1000):
        sc, raw = scenes[0], raws[0]
        s, grp = e.detectMultiScale(sc, 1920, 1080, 1920, 1.25, 2, 24, lim)
        assert s == 0 and grp.tobytes() == oracle.group_first_order(raw[:lim], 2, 0.2).tobytes(), lim
    s, outs = e.detectBatch(scenes, minNeighbors=3, capPerImage=20000)
    assert s == 0
    for raw, got in zip(raws, outs):
        assert got.tobytes() == oracle.group_first_order(raw, 3, 0.2).tobytes()
    k = e.lastStats()
    assert k["phaseMs"]["grouping"] > 0.0 and k["hostMs"]["post"] < 50.0


def test_detect_device_image_and_strides(cuda, vj, oracle, basic_pool, gin):
    torch = cuda
    st, sg = gin["det_stumps"], gin["det_stages"]
    scene = gin["det_scene_1"]
    h, w = scene.shape
    padded = np.zeros((h, w + 13), np.uint8)
    padded[:, :w] = scene
    e = detector(vj, basic_pool, st, sg, norm=1)
    s1, a = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    s2, b = e.detectMultiScale(dev(torch, padded), w, h, w + 13, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s1 == 0 and s2 == 0 and a.tobytes() == b.tobytes()


def test_detect_batch_equals_single(cuda, vj, basic_pool):
    st, sg = vj.synth_cascade(2)
    rng = np.random.default_rng(3)
    scenes = []
    for k in range(6):
        t = rng.random()
        w, h = int(320 * 12 ** t), int(240 * 9 ** t)
        scenes.append(vj.synth_scene(50 + k, min(w, 1280), min(h, 720), 5, 24, 200))
    e = detector(vj, basic_pool, st, sg)
    s, batch = e.detectBatch(scenes, capPerImage=20000)
    assert s == 0
    for sc, b in zip(scenes, batch):
        s, one = e.detectMultiScale(sc, sc.shape[1], sc.shape[0], sc.shape[1], 1.25, 4, 24, 200000)
        assert s == 0 and one.tobytes() == b.tobytes()


def test_detect_rejects_bad_input(cuda, vj, basic_pool, gin):
    e = vj.FaceVisionEngine((24, 24), 1, 64, 64, False, 1000)
    img = np.zeros((32, 32), np.uint8)
    s, _ = e.detectMultiScale(img, 32, 32, 32)
    assert s == vj.Status.kInvalidArg  # no model
    e = detector(vj, basic_pool, gin["det_stumps"], gin["det_stages"], w=64, h=64)
    big = np.zeros((100, 100), np.uint8)
    assert e.detectMultiScale(big, 100, 100, 100)[0] == vj.Status.kInvalidArg
    assert e.detectMultiScale(img, 32, 32, 32, scaleFactor=1.0)[0] == vj.Status.kInvalidArg
    s, d = e.detectMultiScale(np.zeros((20, 20), np.uint8), 20, 20, 20)
    assert s == 0 and len(d) == 0  # smaller than the window: no level


def test_device_grouping_grows_its_scratch(cuda, vj, oracle, basic_pool):
    """A cascade that accepts every window through the variance gate: raw
    detections far outnumber the grouping slots the queue buffers first hold,
    so the launch reports the overflow, the detector grows the queues and
    repeats it, and the grouped result still equals the oracle's."""
    st = np.zeros(1, dtype=vj.STUMP4)
    st[0] = (np.int32(7).view(np.float32), np.float32(0.0), np.float32(1.0), np.float32(1.0))
    sg = np.zeros(1, dtype=vj.STAGE)
    sg[0] = (0, 1, np.float32(-1e30))
    scene = vj.synth_scene(21, 320, 240, 2, 24, 80)
    e = detector(vj, basic_pool, st, sg)
    s, grp = e.detectMultiScale(scene, 320, 240, 320, 1.25, 3, 24, 200000)
    k = e.lastStats()
    assert s == 0 and k["attempts"] >= 2 and k["rawDetections"] > 50000
    ref = oracle.detect(basic_pool, st, sg, scene, threads=8)
    assert len(ref) == k["rawDetections"]
    assert grp.tobytes() == oracle.group_first_order(ref, 3, 0.2).tobytes()
    s, grp2 = e.detectMultiScale(scene, 320, 240, 320, 1.25, 3, 24, 200000)
    assert s == 0 and e.lastStats()["attempts"] == 1 and grp2.tobytes() == grp.tobytes()


def test_crop_resize_batch(cuda, vj, oracle, gin):
    """Device cropResizeTo24 against the reference's outputs (golden), and
    against the oracle for windows of several images in one launch, with
    padded rows and other output sizes."""
    torch = cuda
    img, boxes, out = gin["crop_img"], gin["crop_boxes"], gin["crop_out"]
    dets = np.zeros(len(boxes), dtype=vj.DETECTION)
    for k, (x, y, w, h) in enumerate(boxes):
        dets[k]["x"], dets[k]["y"], dets[k]["w"], dets[k]["h"] = x, y, w, h
    d_img = torch.from_numpy(img).cuda()
    s, patches = vj.crop_resize_batch([d_img], dets, np.zeros(len(boxes), np.int32))
    torch.cuda.synchronize()
    assert s == 0 and np.array_equal(patches.cpu().numpy().reshape(len(boxes), -1), out)
    # several images, one of them a view with padded rows
    scenes = [vj.synth_scene(40 + i, 80 + 37 * i, 60 + 23 * i, 1, 24, 50) for i in range(3)]
    padded = torch.zeros((scenes[1].shape[0], scenes[1].shape[1] + 29), dtype=torch.uint8, device="cuda")
    padded[:, : scenes[1].shape[1]] = torch.from_numpy(scenes[1]).cuda()
    dev = [torch.from_numpy(scenes[0]).cuda(), padded[:, : scenes[1].shape[1]], torch.from_numpy(scenes[2]).cuda()]
    rng = np.random.default_rng(3)
    n = 300
    image_of = rng.integers(0, 3, n).astype(np.int32)
    dets = np.zeros(n, dtype=vj.DETECTION)
    for k in range(n):
        H, W = scenes[image_of[k]].shape
        dets[k]["x"], dets[k]["y"] = rng.integers(-10, W), rng.integers(-10, H)
        dets[k]["w"], dets[k]["h"] = rng.integers(0, 2 * W), rng.integers(0, 2 * H)
    for size in (24, 19):
        s, patches = vj.crop_resize_batch(dev, dets, image_of, out_size=size)
        torch.cuda.synchronize()
        got = patches.cpu().numpy()
        assert s == 0
        for k in range(n):
            b = (dets[k]["x"], dets[k]["y"], dets[k]["w"], dets[k]["h"])
            assert np.array_equal(got[k], oracle.crop_resize(scenes[image_of[k]], b, out=size)), (size, k)
    s, _ = vj.crop_resize_batch(dev, dets[:1], np.array([5], np.int32))
    assert s == vj.Status.kInvalidArg


def test_stage_gate_queues_a_stage_without_reads(cuda, vj, oracle, basic_pool):
    """Rounds queued behind the trainer's stage gate (vj_trainer_set_stage_gate)
    equal rounds run one by one with a read after each, up to the round that
    meets the stage targets; the gate then reads 1 and every queued round
    after it leaves weights, scores, used mask and records untouched."""
    torch = cuda
    npos = nneg = 400
    p = vj.synth_patches(17, npos, nneg)
    labels = np.array([1] * npos + [-1] * nneg, np.int8)
    w0 = np.where(labels > 0, np.float32(0.5) / np.float32(npos), np.float32(0.5) / np.float32(nneg))
    w0 = (w0.astype(np.float64) / w0.astype(np.float64).sum()).astype(np.float32)
    feats = np.ascontiguousarray(basic_pool[:30000])
    rounds = 12
    hit, fa = 0.995, 0.5

    def run(gated):
        T = Train(cuda, vj, oracle, p, labels, feats, w0)
        assert T.t.prepareStage() == 0
        weak = torch.full((rounds, 7), -1, dtype=torch.int32, device="cuda")
        calib = torch.zeros((rounds, 8), dtype=torch.int32, device="cuda")
        gate = torch.zeros(1, dtype=torch.int32, device="cuda")
        h = T.t._h
        if gated:
            assert vj._capi.status("vj_trainer_set_stage_gate", h, gate.data_ptr()) == 0
        snaps = []
        for r in range(rounds):
            assert vj._capi.status("vj_stump_search", h, T.used.data_ptr(), T.best.data_ptr(), None) == 0
            assert vj._capi.status("vj_round_update", h, T.best.data_ptr(), T.strong.data_ptr(), T.used.data_ptr(),
                                 weak[r].data_ptr(), None) == 0
            assert vj._capi.status("vj_stage_calibrate", h, T.strong.data_ptr(), npos, C.c_float(hit), C.c_float(fa),
                                 nneg, calib[r].data_ptr(), None) == 0
            if not gated:
                snaps.append((T.w.cpu().numpy().copy(), T.strong.cpu().numpy().copy(), T.used.cpu().numpy().copy()))
        torch.cuda.synchronize()
        if gated:
            snaps.append((T.w.cpu().numpy().copy(), T.strong.cpu().numpy().copy(), T.used.cpu().numpy().copy()))
        return weak.cpu().numpy(), calib.cpu().numpy(), snaps, int(gate.cpu().item())

    wa, ca, sa, _ = run(False)
    sat = [r for r in range(rounds) if ca[r].view(vj.STAGE_CALIB)[0]["satisfied"]]
    assert sat and sat[0] < rounds - 1  # the targets are met before the last queued round
    k = sat[0]
    wb, cb, sb, g = run(True)
    assert g == 1
    assert np.array_equal(wb[: k + 1], wa[: k + 1]) and np.array_equal(cb[: k + 1], ca[: k + 1])
    assert (wb[k + 1:] == -1).all() and (cb[k + 1:] == 0).all()
    for x, y in zip(sb[0], sa[k]):
        assert np.array_equal(x, y)


def test_last_round_reports_pick_and_runner_up(cuda, vj, oracle, gin, basic_pool):
    """vj_trainer_last_round: the pick's exact error and feature equal the
    search's output, and the runner-up among the exactly replayed candidates is
    the oracle's second-best stump (the best of the pool with the pick masked),
    up to features whose errors lie within the candidate window of it."""
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    rng = np.random.default_rng(12)
    w = (rng.random(320) / 320).astype(np.float32)
    feats = np.ascontiguousarray(basic_pool[:20000])
    T = Train(cuda, vj, oracle, patches, labels, feats, w)
    sums, inv = oracle.train_integrals(patches)
    of = np.ascontiguousarray(feats).view(oracle.FEATURE)
    for _ in range(3):
        f, e, th, par = T.search(used=True)
        info = T.t.lastRound()
        assert info["bestFeature"] == f and np.float32(info["bestErr"]) == np.float32(e)
        assert info["candidates"] >= 1 and info["status"] == 0
        used = T.used.cpu().numpy().copy()
        used[f] = 1
        ru = oracle.weak_search(of, sums, inv, labels, T.w.cpu().numpy(), used=used, threads=8)
        if info["runnerUpFeature"] >= 0:
            assert info["runnerUpErr"] >= ru["err"] and info["runnerUpErr"] - ru["err"] <= info["window"]
            if info["runnerUpErr"] == ru["err"]:
                assert info["runnerUpFeature"] == ru["featureIdx"]
        else:
            assert ru["err"] > info["fastMin"]  # every other feature lay outside the window
        assert T.t.applyBestWeak(T.best, T.strong, T.used) == 0


def test_tilted_features_like_the_reference(cuda, vj, oracle, golden, gin):
    """The device search and detection over tilted (All-mode) features give the
    reference's picks and raw detections (corner indices on the upright
    integral, as the reference evaluates them), and the reference's clusters."""
    allp = oracle.feature_pool(2)
    patches = gin["ws_patches"]
    labels = np.array([1] * 160 + [-1] * 160, np.int8)
    for g in golden["tilted_weak_search"]:
        T = Train(cuda, vj, oracle, patches, labels, np.ascontiguousarray(allp[gin[g["key"] + "_idx"]]),
                  gin[g["key"] + "_w"])
        assert T.search() == (g["featureIdx"], f32(g["err_bits"]), f32(g["theta_bits"]), g["parity"]), g
    e = vj.FaceVisionEngine((24, 24), 1, 640, 480, False, 200000)
    assert e.setCascadeModel(allp.view(vj.HAAR_FEATURE), gin["tdet_stumps"].view(vj.STUMP4),
                             gin["tdet_stages"].view(vj.STAGE)) == 0
    scene = gin["tdet_scene"]
    s, raw = e.detectMultiScale(scene, 200, 150, 200, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and raw.tobytes() == gin["tdet_raw"].tobytes()
    s, grp = e.detectMultiScale(scene, 200, 150, 200, 1.25, 4, 24, 200000)
    assert s == 0 and as_set(grp) == as_set(gin["tdet_grouped"])
    assert grp.tobytes() == oracle.group_first_order(raw, 4, 0.2).tobytes()


# ---------------------------------------------------------------- sweep pruning
def test_pruned_sweep_rounds_equal_oracle_and_fresh_searches(cuda, vj, oracle, basic_pool):
    """Within a stage the sweep skips features whose error bound (last round's
    error times the update's factor) cannot reach the candidate window.  Ten
    rounds with the resident orders: every pick equals the oracle's and that
    of a fresh search (a new bind, so nothing is pruned), and some round
    actually skips features.  Weights edited outside vj_round_update between
    two rounds turn the pruning off for that round (the pick still equals the
    oracle's), as does clearing a used-mask entry."""
    torch = cuda
    npos = nneg = 2000
    p = vj.synth_patches(71, npos, nneg)
    labels = np.array([1] * npos + [-1] * nneg, np.int8)
    feats = np.ascontiguousarray(basic_pool[::7])
    n, F = len(labels), len(feats)
    w0 = np.full(n, np.float32(0.5) / np.float32(npos), np.float32)
    T = Train(cuda, vj, oracle, p, labels, feats, w0)
    assert T.t.prepareStage() == 0
    sums, inv = oracle.train_integrals(p)
    used = np.zeros(F, np.uint8)
    weak = cuda.zeros(7, dtype=cuda.int32, device="cuda")
    swept = []
    rng = np.random.default_rng(5)
    for r in range(10):
        if r == 6:  # an edit outside the round update
            w = T.w.cpu().numpy() * (1.0 + 0.01 * rng.random(n)).astype(np.float32)
            T.w.copy_(torch.from_numpy((w / w.sum(dtype=np.float64)).astype(np.float32)))
        if r == 8:  # a used feature cleared again
            f_clear = int(np.nonzero(used)[0][0])
            used[f_clear] = 0
            T.used[f_clear] = 0
        got = T.search(used=True)
        swept.append(T.t.lastRound()["swept"])
        w = T.w.cpu().numpy()
        ref = oracle.weak_search(feats, sums, inv, labels, w, used=used, threads=16)
        assert got == (ref["featureIdx"], ref["err"], ref["theta"], ref["parity"]), r
        fresh = Train(cuda, vj, oracle, p, labels, feats, w)
        assert fresh.t.prepareStage() == 0
        fresh.used.copy_(T.used)
        assert fresh.search(used=True) == got, r
        assert fresh.t.lastRound()["swept"] == F - int(used.sum())  # a fresh bind prunes nothing
        assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
        used[got[0]] = 1
    assert swept[0] == F  # the first search of a stage has no bounds yet
    assert swept[6] == F - 6  # the edited weights: every unused feature streamed
    assert min(swept[1:6]) < F // 2, swept  # bounds skip most features in some round
