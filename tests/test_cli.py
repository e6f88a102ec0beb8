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
