"""Detection engine: launch shapes, the autotuner and the work counters.

Every launch shape (tile rows, tile-pass depth, lane-per-window queue passes,
CTAs per SM) must give the raw detections of the oracle's restatement of
detectMultiScaleCpu (src/main.cu:684-827) bit for bit; the autotuner checks
the same across its candidates and keeps one of them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = [
    dict(tileRows=8, tileStumps=64, queueStumps=0, blocksPerSM=4, deepSlots=2),
    dict(tileRows=4, tileStumps=1, queueStumps=0, blocksPerSM=0, deepSlots=1),
    dict(tileRows=16, tileStumps=111, queueStumps=0, blocksPerSM=0, deepSlots=2),
    dict(tileRows=8, tileStumps=36, queueStumps=400, blocksPerSM=0, deepSlots=1),
    dict(tileRows=8, tileStumps=11, queueStumps=2000, blocksPerSM=2, deepSlots=2),
    dict(tileRows=4, tileStumps=100000, queueStumps=0, blocksPerSM=1, deepSlots=2),
    dict(tileRows=16, tileStumps=61, queueStumps=0, blocksPerSM=4, deepSlots=1),
]


@pytest.fixture(scope="module")
def full_case(vj, oracle, basic_pool):
    st, sg = vj.synth_cascade(2)
    scene = vj.synth_scene(7, 800, 600, 12, 24, 200)
    ref = oracle.detect(basic_pool, st, sg, scene, norm_mode=0, threads=8)
    return st, sg, scene, ref


def engine(vj, pool, st, sg, maxdet=200000):
    e = vj.FaceVisionEngine((24, 24), 1, 3840, 2160, False, maxdet)
    assert e.setCascadeModel(pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4), sg.view(vj.STAGE)) == 0
    return e


@pytest.mark.parametrize("cfg", CONFIGS, ids=[f"th{c['tileRows']}-t{c['tileStumps']}-q{c['queueStumps']}-b"
                                              f"{c['blocksPerSM']}-s{c['deepSlots']}" for c in CONFIGS])
def test_every_launch_shape_matches_oracle(cuda, vj, basic_pool, full_case, cfg):
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    assert e.setConfig(**cfg) == 0
    assert e.getConfig() == cfg
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0
    assert len(raw) == len(ref) and raw.tobytes() == ref.tobytes()
    stats = e.lastStats()
    assert stats["rawDetections"] == len(ref)
    assert stats["queuePasses"] == (0 if cfg["queueStumps"] == 0 else stats["queuePasses"])


def test_bad_config_rejected(cuda, vj, basic_pool, full_case):
    st, sg, _, _ = full_case
    e = engine(vj, basic_pool, st, sg)
    assert e.setConfig(tileRows=5) == vj.Status.kInvalidArg
    assert e.setConfig(tileStumps=-1) == vj.Status.kInvalidArg
    assert e.setConfig(deepSlots=3) == vj.Status.kInvalidArg
    assert e.getConfig()["tileRows"] == 8


def test_stats_are_consistent(cuda, vj, basic_pool, full_case):
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0
    k = e.lastStats()
    assert k["images"] == 1 and k["levels"] > 5
    assert k["windows"] >= k["gated"] > 0
    assert k["stumpEvals"] >= k["gated"]
    assert k["rawDetections"] == len(raw) == len(ref)
    assert k["attempts"] >= 1 and k["gpuMs"] > 0
    assert all(v >= 0 for v in k["phaseMs"].values())
    assert k["deepWindows"] >= k["rawDetections"]


def test_small_capacity_grows_and_repeats(cuda, vj, basic_pool, full_case):
    """maxDetections 20 starts the per-image buffer at 64 entries; the
    overflow is seen, the buffer grows and the launch repeats, and the result
    is the oracle's list truncated to 20."""
    st, sg, scene, ref = full_case
    assert len(ref) > 64
    e = engine(vj, basic_pool, st, sg, maxdet=20)
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 20, applyGrouping=False)
    assert s == 0 and e.lastStats()["attempts"] >= 2
    assert raw.tobytes() == ref[:20].tobytes()


def test_autotune_keeps_identical_results(cuda, vj, basic_pool, full_case):
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    scenes = [scene, vj.synth_scene(8, 640, 480, 4, 24, 200), vj.synth_scene(9, 320, 240, 2, 24, 100)]
    s, cfg, ms = e.autotune(scenes, repeats=1)
    assert s == 0 and ms > 0
    assert cfg["tileRows"] in (4, 8, 16) and cfg["deepSlots"] in (1, 2) and cfg == e.getConfig()
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and raw.tobytes() == ref.tobytes()


def test_batch_on_device_images(cuda, vj, basic_pool, full_case):
    torch = cuda
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    others = [vj.synth_scene(20 + k, 200 + 97 * k, 150 + 61 * k, 2, 24, 120) for k in range(5)]
    imgs = [scene] + others
    dev = [torch.from_numpy(im).cuda() for im in imgs]
    s, host_res = e.detectBatch(imgs, applyGrouping=False, capPerImage=20000)
    s2, dev_res = e.detectBatch(dev, applyGrouping=False, capPerImage=20000)
    assert s == 0 and s2 == 0
    assert host_res[0].tobytes() == ref.tobytes()
    for a, b in zip(host_res, dev_res):
        assert a.tobytes() == b.tobytes()


def test_batch_host_copy_forms(cuda, vj, basic_pool, full_case):
    """Host images reach the device by one contiguous copy (page-locked, stride
    a multiple of 16), row by row, or gathered into a pinned buffer by host
    threads (16 MB or more of images that are not contiguous copies): the
    three forms give the results of the same images on the device."""
    torch = cuda
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    sizes = [(1920, 1080), (1283, 721), (1600, 912), (1001, 1333), (2048, 1152), (1440, 999), (1920, 1080),
             (1111, 777), (3840, 2160)]
    imgs = [scene] + [vj.synth_scene(40 + k, w, h, 3, 24, 200) for k, (w, h) in enumerate(sizes)]
    assert sum(im.size for im in imgs) >= 16 << 20
    dev = [torch.from_numpy(im).cuda() for im in imgs]
    s0, want = e.detectBatch(dev, applyGrouping=False, capPerImage=20000)
    assert s0 == 0 and want[0].tobytes() == ref.tobytes()
    keep = [torch.from_numpy(im).pin_memory() for im in imgs]
    pinned = [t.numpy() for t in keep]
    # pageable, >= 16 MB: gathered; page-locked: contiguous copies where the
    # width is a multiple of 16, row by row for the rest (below 16 MB)
    for batch in (imgs, pinned, pinned[:3] + imgs[3:5], imgs[:2]):
        s, got = e.detectBatch(batch, applyGrouping=False, capPerImage=20000)
        assert s == 0
        for a, b in zip(got, want):
            assert a.tobytes() == b.tobytes()


def test_large_batch_column_walk(cuda, vj, basic_pool, full_case):
    """A batch with enough 32-column chunks (56 scenes of 1920x1080, about
    17,700 chunks) takes the integral column pass as one walk per chunk down
    all rows; each image alone takes the segment passes.  Same detections."""
    st, sg, _, _ = full_case
    e = engine(vj, basic_pool, st, sg)
    imgs = [vj.synth_scene(300 + k, 1920, 1080, 4, 24, 200) for k in range(56)]
    s, batch = e.detectBatch(imgs, applyGrouping=False, capPerImage=20000)
    assert s == 0
    for im, got in zip(imgs[::5], batch[::5]):
        s1, alone = e.detectMultiScale(im, 1920, 1080, 1920, 1.25, 4, 24, 200000, applyGrouping=False)
        assert s1 == 0 and alone.tobytes() == got.tobytes()


def test_reserved_arena(cuda, vj, basic_pool, full_case):
    """With a reserved arena every batch is laid out inside it: same results,
    the detector holds no more than the reservation (plus the model and the
    plan), and a batch that does not fit is refused."""
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    assert e.reserve(512 << 20) == 0
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and raw.tobytes() == ref.tobytes()
    assert (512 << 20) <= e.deviceBytes() < (512 << 20) + (8 << 20)
    assert e.reserve(1 << 20) == 0
    s, _ = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == vj.Status.kOutOfMemory
    assert e.reserve(0) == 0  # back to buffers grown on demand
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and raw.tobytes() == ref.tobytes()


def test_barrier_wait_runs_out_and_context_survives(cuda, vj, basic_pool, full_case):
    """A grid-barrier wait that cannot finish (one block leaves before the
    first barrier) ends after its short limit with VJ_RUNTIME_ERROR; the next
    launch on the same context gives the oracle's detections."""
    import time
    st, sg, scene, ref = full_case
    e = engine(vj, basic_pool, st, sg)
    lib = vj.load()
    h, w = scene.shape
    assert lib.vj_detector_test_barrier_timeout(e._h, 5, 2_000_000) == 0
    t0 = time.time()
    s, _ = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == vj.Status.kRuntimeError and time.time() - t0 < 30
    assert b"barrier" in lib.vj_last_error()
    assert lib.vj_detector_test_barrier_timeout(e._h, -1, 0) == 0
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0 and raw.tobytes() == ref.tobytes()


def _stage_sums(pool, st, sg, scene, oracle, last):
    """The reference's FP32 stage sums (stumps added in order from 0.0f) of
    every full-size window of the image, stages 0..last, with the survivors of
    each stage; restated from detectMultiScaleCpu (src/main.cu:755-819) on the
    first pyramid level (the image itself, step 1)."""
    s, q = oracle.integral(scene)
    S = s.astype(np.int64).ravel()
    Q = q.astype(np.uint64).ravel()
    h, w = scene.shape
    P = w + 1
    ys, xs = np.mgrid[0:h - 23, 0:w - 23]
    b = (ys * P + xs).ravel()
    o = [P + 1, P + 23, 23 * P + 1, 23 * P + 23]
    ns = (S[b + o[0]] - S[b + o[1]] - S[b + o[2]] + S[b + o[3]]).astype(np.float64)
    m32 = np.uint64(0xFFFFFFFF)
    qq = ((Q[b + o[0]] - Q[b + o[1]] - Q[b + o[2]] + Q[b + o[3]]) & m32).astype(np.float64)
    nf2 = 484.0 * qq - ns * ns
    inv = np.zeros(len(b), np.float32)
    pos = nf2 > 0
    inv[pos] = (1.0 / np.sqrt(nf2[pos])).astype(np.float32)
    alive = np.nonzero(pos & (484.0 * inv.astype(np.float64) < 0.1))[0]
    fidx = st["featureBits"].view(np.int32)
    out = []
    for k in range(last + 1):
        f0, nt, thr = int(sg[k]["first"]), int(sg[k]["ntrees"]), np.float32(sg[k]["threshold"])
        bb = b[alive]
        acc = np.zeros(len(alive), np.float32)
        for j in range(nt):
            ft = pool[fidx[f0 + j]]
            raw = np.zeros(len(alive), np.float32)
            for ri, r in enumerate(("r0", "r1", "r2")[:int(ft["rectCount"])]):
                c = [S[bb + (int(ft[r][p]) // 25) * P + int(ft[r][p]) % 25].astype(np.float32)
                     for p in ("p0", "p1", "p2", "p3")]
                v = (((c[0] - c[1]) - c[2]) + c[3]) * np.float32(ft[r]["w"])
                raw = v if ri == 0 else (raw + v)
            resp = raw * inv[alive]
            acc = acc + np.where(resp < st["theta"][f0 + j], st["leftVal"][f0 + j], st["rightVal"][f0 + j])
        out.append((alive.copy(), acc))
        alive = alive[~(acc < thr)]
    return out


def test_deep_stage_sums_on_the_threshold(cuda, vj, oracle, basic_pool):
    """Deep-pass stages decide from order-free sums and replay a stage with the
    sequential FP32 sum when the total is within the stage's tolerance of its
    threshold.  Thresholds placed exactly on a window's sequential sum (which
    passes: !(acc < threshold)) and one ulp above another window's sum (which
    fails) must give the oracle's detections."""
    st, sg = vj.synth_cascade(2)
    sg = sg.copy()
    scene = vj.synth_scene(21, 160, 120, 2, 24, 60)
    e = engine(vj, basic_pool, st, sg)
    deep_from = 5  # stages 0-4 (111 stumps) run in the tile pass with the default config
    for k in (deep_from, deep_from + 1, deep_from + 2):
        sums = _stage_sums(basic_pool, st, sg, scene, oracle, k)
        alive, acc = sums[k]
        assert len(alive) > 4, k
        order = np.argsort(acc)
        pick = acc[order[len(order) // 3]]
        # every survivor at or above `pick` passes, the ones below fail
        sg[k]["threshold"] = pick if k != deep_from + 1 else np.nextafter(pick, np.float32(np.inf))
    ref = oracle.detect(basic_pool, st, sg, scene, norm_mode=0, threads=8)
    e = engine(vj, basic_pool, st, sg)
    h, w = scene.shape
    s, raw = e.detectMultiScale(scene, w, h, w, 1.25, 4, 24, 200000, applyGrouping=False)
    assert s == 0
    assert len(raw) == len(ref) and raw.tobytes() == ref.tobytes()
