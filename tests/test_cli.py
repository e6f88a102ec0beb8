"""Command-line drop-ins: vj_detect takes `cuda_hello detect`'s arguments
(src/main.cu:2394-2579) and writes the same PPM."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
EXE = ROOT / "cs677s26_gb300" / "bin" / "vj_detect"


def write_pgm(path, img, comment=True):
    h, w = img.shape
    head = b"P5\n" + (b"# synthetic scene\n" if comment else b"") + f"{w} {h}\n255\n".encode()
    path.write_bytes(head + img.tobytes())


def read_ppm(path):
    data = path.read_bytes()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6"
    w, h = map(int, parts[1].split())
    assert parts[2] == b"255"
    return np.frombuffer(parts[3], np.uint8).reshape(h, w, 3)


def frames(img, dets):
    """The reference's drawRect: 2-pixel white frames, clipped."""
    h, w = img.shape
    rgb = np.repeat(img[:, :, None], 3, axis=2).copy()
    for d in dets:
        x0, y0 = max(0, d["x"]), max(0, d["y"])
        x1, y1 = min(w - 1, d["x"] + d["w"] - 1), min(h - 1, d["y"] + d["h"] - 1)
        if x0 > x1 or y0 > y1:
            continue
        for t in range(2):
            rgb[min(h - 1, y0 + t), x0:x1 + 1] = 255
            rgb[max(0, y1 - t), x0:x1 + 1] = 255
            rgb[y0:y1 + 1, min(w - 1, x0 + t)] = 255
            rgb[y0:y1 + 1, max(0, x1 - t)] = 255
    return rgb


@pytest.fixture(scope="module")
def model_file(vj, basic_pool, tmp_path_factory):
    st, sg = vj.synth_cascade(2)
    p = tmp_path_factory.mktemp("model") / "cascade_model.bin"
    assert vj.ModelIO.saveCascadeModel(str(p), (24, 24), basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4),
                                       sg.view(vj.STAGE))
    return p, st, sg


def test_usage_and_bad_inputs(vj, model_file, tmp_path):
    r = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage: vj_detect" in r.stderr
    r = subprocess.run([str(EXE), str(tmp_path / "missing.bin"), "a.pgm", "b.ppm"], capture_output=True, text=True)
    assert r.returncode == 1 and "loadCascadeModel failed" in r.stderr
    bad = tmp_path / "bad.pgm"
    bad.write_bytes(b"P2\n2 2\n255\n0 0 0 0\n")
    r = subprocess.run([str(EXE), str(model_file[0]), str(bad), str(tmp_path / "o.ppm")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "need P5" in r.stderr


@pytest.mark.gpu
def test_vj_detect_writes_the_reference_image(cuda, vj, basic_pool, model_file, tmp_path):
    path, st, sg = model_file
    scene = vj.synth_scene(5, 640, 480, 6, 24, 200)
    pgm, ppm = tmp_path / "in.pgm", tmp_path / "out.ppm"
    write_pgm(pgm, scene)
    r = subprocess.run([str(EXE), str(path), str(pgm), str(ppm), "1.25", "4", "24", "200000"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "[DETECT] detections=" in r.stdout and "[OK] Saved result to:" in r.stdout
    e = vj.FaceVisionEngine((24, 24), 1, 640, 480, False, 200000)
    assert e.setCascadeModel(basic_pool.view(vj.HAAR_FEATURE), st.view(vj.STUMP4), sg.view(vj.STAGE)) == 0
    s, dets = e.detectMultiScale(scene, 640, 480, 640)
    assert s == 0 and f"detections={len(dets)}" in r.stdout
    assert np.array_equal(read_ppm(ppm), frames(scene, dets))
    r = subprocess.run([str(EXE), str(path), str(pgm), str(ppm), "1.25", "4", "24", "200000", "2"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[DETECT_BENCH] runs=2" in r.stdout


TRAIN = ROOT / "cs677s26_gb300" / "bin" / "vj_train"


def test_vj_train_arguments(tmp_path):
    r = subprocess.run([str(TRAIN)], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage: vj_train" in r.stderr
    r = subprocess.run([str(TRAIN), str(tmp_path / "m.bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "stageNegCacheDir is required" in r.stderr
    args = [str(tmp_path / "faces.bin"), "10000", "250", "200000", "4", "1.0", str(tmp_path / "m.bin")]
    r = subprocess.run([str(TRAIN)] + args, capture_output=True, text=True)
    assert r.returncode == 1 and "scaleFactor must be > 1.0" in r.stderr
    (tmp_path / "faces.bin").write_bytes(bytes(100))
    args = [str(tmp_path / "faces.bin"), "10000", "250", "200000", "4", "1.25", "38", "0.99", "0.4", "24",
            str(tmp_path), str(tmp_path), "677", "3", str(tmp_path / "m.bin")]
    r = subprocess.run([str(TRAIN)] + args, capture_output=True, text=True)
    assert r.returncode == 1 and "not divisible by samplePixels" in r.stderr


@pytest.mark.gpu
def test_vj_train_small_cascade(cuda, vj, oracle, tmp_path):
    """A short training run on synthetic data: the stage-0 training set it
    dumps gives, through the oracle's restatement of runCpuWeakSearch over the
    Core pool, the first weak classifier the run reports; the saved model
    loads and detects."""
    faces = vj.synth_patches(11, 2000, 0)
    (tmp_path / "faces.bin").write_bytes(faces.tobytes())
    negdir = tmp_path / "neg"
    negdir.mkdir()
    for k in range(24):
        write_pgm(negdir / f"n{k:02d}.pgm", vj.synth_scene(700 + k, 320 + 16 * k, 240 + 8 * k, 0, 24, 100))
    dump = tmp_path / "dump"
    dump.mkdir()
    model = tmp_path / "model.bin"
    args = [str(tmp_path / "faces.bin"), "10000", "4", "200000", "4", "1.25", "3", "0.95", "0.8", "24",
            str(tmp_path), str(negdir), "677", "3", str(model)]
    env = dict(__import__("os").environ, VJ_TRAIN_DUMP=str(dump))
    r = subprocess.run([str(TRAIN)] + args, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "[OK] Saved model to:" in r.stdout
    first = [ln for ln in r.stdout.splitlines() if ln.startswith("[TRAIN] stage=0 weak=0 ")][0]
    fields = dict(kv.split("=", 1) for kv in first.split()[1:] if "=" in kv)
    # stage 0 set: 2000 positives then 10000 negatives, weights 0.5/n normalised
    raw = np.frombuffer((dump / "stage00.bin").read_bytes(), np.uint8).reshape(-1, 24, 24)
    assert raw.shape[0] == 12000 and np.array_equal(raw[:2000], faces)
    labels = np.array([1] * 2000 + [-1] * 10000, np.int8)
    w = np.where(labels > 0, np.float32(0.5) / np.float32(2000), np.float32(0.5) / np.float32(10000))
    w = (w.astype(np.float64) / w.astype(np.float64).sum()).astype(np.float32)
    sums, inv = oracle.train_integrals(raw)
    core = np.ascontiguousarray(vj.feature_pool(vj.FeatureMode.Core)).view(oracle.FEATURE)
    best = oracle.weak_search(core, sums, inv, labels, w, threads=16)
    assert int(fields["feature"]) == best["featureIdx"]
    assert int(fields["parity"]) == best["parity"]
    feats, stumps, stages = vj.ModelIO.loadCascadeModel(str(model))[1:4]
    assert len(stages) >= 1 and len(feats) == 210400
    pgm, ppm = tmp_path / "s.pgm", tmp_path / "s.ppm"
    write_pgm(pgm, vj.synth_scene(9, 640, 480, 4, 24, 200))
    r = subprocess.run([str(EXE), str(model), str(pgm), str(ppm)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[DETECT] detections=" in r.stdout
