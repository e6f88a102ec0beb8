"""Continuous-batching server (vj_server_*): each request's detections are the
same alone and in the mix, equal to vj_detect on that image by itself
(FaceVisionEngine::detectMultiScale, src/face_vision_engine.cu:1541-1747)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(vj, basic_pool):
    st, sg = vj.synth_cascade(2)
    return basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4), sg.view(vj.STAGE)


@pytest.fixture(scope="module")
def scenes(vj):
    rng = np.random.default_rng(11)
    out = []
    for k in range(24):
        t = rng.random()
        w, h = int(round(320 * 6 ** t)), int(round(240 * 4.5 ** t))
        out.append(vj.synth_scene(300 + k, w, h, 4, 24, 200))
    return out


@pytest.fixture(scope="module")
def alone(vj, model, scenes):
    f, s, g = model
    e = vj.FaceVisionEngine((24, 24), 1, 3840, 2160, False, 200000)
    assert e.setCascadeModel(f, s, g) == 0
    res = []
    for sc in scenes:
        st, d = e.detectMultiScale(sc, sc.shape[1], sc.shape[0], sc.shape[1])
        assert st == 0
        res.append(d)
    return res


def test_results_equal_alone_and_in_the_mix(cuda, vj, model, scenes, alone):
    f, s, g = model
    srv = vj.DetectServer(f, s, g, workers=2, maxBatchImages=8, hbmBudgetBytes=8 << 30)
    try:
        # one request on an idle server
        t = srv.submit(scenes[0])
        st, d = srv.wait(t)
        assert st == 0 and d.tobytes() == alone[0].tobytes()
        # all at once from two submitting threads: they share batches
        tickets = [None] * len(scenes)

        def submit(idx):
            for i in idx:
                tickets[i] = srv.submit(scenes[i])

        th = [threading.Thread(target=submit, args=(range(k, len(scenes), 2),)) for k in range(2)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for i, t in enumerate(tickets):
            st, d = srv.wait(t)
            assert st == 0 and d.tobytes() == alone[i].tobytes(), f"request {i}"
        k = srv.stats()
        assert k["completed"] == k["submitted"] == len(scenes) + 1 and k["failed"] == 0
        assert k["batches"] < k["completed"]  # requests were batched together
        assert 0 < k["p50Ms"] <= k["p99Ms"] <= k["p999Ms"] <= k["maxMs"]
        assert k["peakAdmittedBytes"] <= 8 << 30
        assert k["deviceBytes"] < (8 << 30) + (64 << 20)  # the arenas hold the budget
    finally:
        srv.close()


def test_plain_mode_is_one_image_per_batch(cuda, vj, model, scenes, alone):
    f, s, g = model
    srv = vj.DetectServer(f, s, g, workers=1, maxBatchImages=1, hbmBudgetBytes=4 << 30)
    try:
        tickets = [srv.submit(sc) for sc in scenes[:6]]
        for i, t in enumerate(tickets):
            st, d = srv.wait(t)
            assert st == 0 and d.tobytes() == alone[i].tobytes()
        k = srv.stats()
        assert k["batches"] == 6 and k["meanBatchImages"] == 1.0
    finally:
        srv.close()


def test_admission_by_budget(cuda, vj, model, scenes):
    f, s, g = model
    small = vj.estimate_detect_bytes(320, 240)
    big = vj.estimate_detect_bytes(1920, 1080)
    assert 0 < small < big
    # each worker's share fits a 320x240 image but not a 1080p one
    srv = vj.DetectServer(f, s, g, workers=2, maxBatchImages=64, hbmBudgetBytes=2 * (small * 3))
    try:
        with pytest.raises(vj.VJError) as ei:
            srv.submit(np.zeros((1080, 1920), np.uint8))
        assert ei.value.status == vj.Status.kOutOfMemory
        img = scenes[0][:240, :320].copy()
        tickets = [srv.submit(img) for _ in range(12)]
        for t in tickets:
            st, _ = srv.wait(t)
            assert st == 0
        k = srv.stats()
        assert k["meanBatchImages"] <= 3.0  # the budget caps the batch
        assert k["peakAdmittedBytes"] <= 2 * (small * 3)
    finally:
        srv.close()


def test_poll_wait_and_unknown_ticket(cuda, vj, model, scenes):
    f, s, g = model
    srv = vj.DetectServer(f, s, g, workers=1, maxBatchImages=4, hbmBudgetBytes=2 << 30)
    try:
        t = srv.submit(scenes[1])
        deadline = time.time() + 30
        while not srv.poll(t) and time.time() < deadline:
            time.sleep(0.001)
        assert srv.poll(t)
        st, _ = srv.wait(t, timeoutMs=0)
        assert st == 0
        st, _ = srv.wait(t)  # released
        assert st == vj.Status.kInvalidArg
    finally:
        srv.close()


def test_batch_pixel_cap(cuda, vj, model, scenes, alone):
    """maxBatchPixels: a batch takes requests while their pixels fit the cap (a
    lone larger image still runs), so a cap below every image gives one image
    per batch and a cap of two small images at most two; results unchanged."""
    f, s, g = model
    small = sorted(range(len(scenes)), key=lambda i: scenes[i].size)[:8]
    for cap, most in ((1, 1), (2 * max(scenes[i].size for i in small), 2)):
        srv = vj.DetectServer(f, s, g, workers=1, maxBatchImages=64, maxBatchPixels=cap, hbmBudgetBytes=8 << 30)
        try:
            tickets = [srv.submit(scenes[i]) for i in small]
            for i, t in zip(small, tickets):
                st, d = srv.wait(t)
                assert st == 0 and d.tobytes() == alone[i].tobytes()
            k = srv.stats()
            assert k["completed"] == len(small) and k["batches"] >= len(small) / most
            if most == 1:
                assert k["batches"] == len(small)
        finally:
            srv.close()
