"""A small training run end to end: 2,000 + 2,000 patches (seed 677), a 3-stage cascade
trained in the run on the device (1, 2 and 3 rounds over the full 162,336
Basic pool; main.cu:1955-2348), then integral images of a 640x480 scene with 3
pasted faces and single-scale detection with that cascade.  Every stump pick,
stage threshold, integral and detection is compared with the oracle."""
import numpy as np
import pytest

from test_gpu_parity import Train, dev

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_three_stage_training_and_single_scale_detect(cuda, vj, oracle, basic_pool):
    torch = cuda
    npos = nneg = 2000
    p = vj.synth_patches(677, npos, nneg)
    labels = np.array([1] * npos + [-1] * nneg, np.int8)
    w0 = np.where(labels > 0, np.float32(0.5) / np.float32(npos), np.float32(0.5) / np.float32(nneg))
    w0 = (w0.astype(np.float64) / w0.astype(np.float64).sum()).astype(np.float32)
    T = Train(cuda, vj, oracle, p, labels, basic_pool, w0)
    assert T.t.prepareStage() == 0
    sums, inv = oracle.train_integrals(p)
    feats = np.ascontiguousarray(basic_pool).view(oracle.FEATURE)
    weak = torch.zeros(7, dtype=torch.int32, device="cuda")
    calib = torch.zeros(8, dtype=torch.int32, device="cuda")
    stumps, stages = [], []
    for nrounds in (1, 2, 3):
        T.w.copy_(torch.from_numpy(w0))
        T.strong.zero_()
        T.used.zero_()
        used = np.zeros(len(basic_pool), np.uint8)
        strong = np.zeros(len(labels), np.float32)
        first = len(stumps)
        for _ in range(nrounds):
            got = T.search(used=True)
            w = T.w.cpu().numpy()
            ref = oracle.weak_search(feats, sums, inv, labels, w, used=used, threads=16)
            assert got == (ref["featureIdx"], ref["err"], ref["theta"], ref["parity"])
            assert T.t.applyBestWeak(T.best, T.strong, T.used, weak) == 0
            wr = w.copy()
            oracle.round_update(feats, dict(featureIdx=got[0], err=got[1], theta=got[2], parity=got[3]), sums, inv,
                                labels, wr, strong)
            gw = T.w.cpu().numpy()
            assert np.max(np.abs(gw.view(np.int32).astype(np.int64) - wr.view(np.int32).astype(np.int64))) <= 1
            assert np.array_equal(T.strong.cpu().numpy(), strong)
            used[got[0]] = 1
            wk = weak.cpu().numpy().view(vj.WEAK)[0]
            stumps.append((np.int32(wk["featureIdx"]).view(np.float32), wk["theta"], wk["leftVal"], wk["rightVal"]))
        assert T.t.calibrateStage(T.strong, npos, 0.99, 0.4, nneg, calib) == 0
        cal = calib.cpu().numpy().view(vj.STAGE_CALIB)[0]
        refc = oracle.stage_calibrate(strong, npos, np.float32(0.99), np.float32(0.4), nneg)
        assert np.float32(cal["stageThreshold"]).tobytes() == np.float32(refc["stageThreshold"]).tobytes()
        stages.append((first, nrounds, np.float32(cal["stageThreshold"]) - np.float32(1e-5)))
    st = np.array(stumps, dtype=np.float32).view(vj.STUMP4).reshape(-1)
    sg = np.zeros(len(stages), dtype=vj.STAGE)
    for i, (f_, n_, t_) in enumerate(stages):
        sg[i] = (f_, n_, t_)

    # the scene's integral images
    scene = vj.synth_scene(677, 640, 480, 3, 24, 120)
    d_img = dev(torch, scene)
    d_sum = torch.zeros(481 * 641, dtype=torch.int32, device="cuda")
    d_sq = torch.zeros(481 * 641, dtype=torch.int64, device="cuda")
    vj._capi.call("vj_integral_image", d_img.data_ptr(), 640, 480, 640, d_sum.data_ptr(), d_sq.data_ptr(), None)
    rs, rq = oracle.integral(scene)
    assert np.array_equal(d_sum.cpu().numpy().view(np.uint32), rs.reshape(-1).view(np.uint32))
    assert np.array_equal(d_sq.cpu().numpy().view(np.uint64), rq.reshape(-1).view(np.uint64))

    # single-scale detection: scaleFactor 27 leaves only level 0 (480 / 27 < 24)
    e = vj.FaceVisionEngine((24, 24), 1, 640, 480, False, 200000)
    assert e.setCascadeModel(basic_pool.view(vj.HAAR_FEATURE), st, sg) == 0
    s, raw = e.detectMultiScale(scene, 640, 480, 640, 27.0, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and e.lastStats()["levels"] == 1
    ref = oracle.detect(basic_pool, st, sg, scene, sf=27.0, threads=16)
    assert len(raw) == len(ref) and raw.tobytes() == ref.tobytes()
