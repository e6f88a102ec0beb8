"""The full stage training step (10,000 face + 10,000 texture patches of seed
1, all 162,336 Basic features, uniform initial weights, 50 rounds of search,
FP64 round update and stage calibration) on the device, against
tests/golden/stage_step_picks.json: the oracle's restatement of the reference's
runCpuWeakSearch (main.cu:587-682) over the same rounds, some of which
make_stage_step_picks.py also checked against the reference's own function.

Every round's pick (featureIdx, FP32 error, theta, parity) must equal the
fixture's bit for bit, and so must every calibration.  The FP64 update may
differ from the oracle's in the last bit of a weight (CUDA's double exp/log
against the C library's), so the weights are checked per round by hash and,
at the end, to within one unit in the last place; the strong scores depend
only on the picks and must be equal."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, f32bits

pytestmark = pytest.mark.gpu


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_stage_step_fifty_picks_equal_the_oracle(cuda, vj):
    torch = cuda
    g = json.loads((GOLDEN / "stage_step_picks.json").read_text())
    final = np.load(GOLDEN / "stage_step_final.npz")
    npos, nneg = g["npos"], g["nneg"]
    p = vj.synth_patches(g["seed"], npos, nneg)
    assert sha(p) == g["patches_sha256"]
    pool = vj.feature_pool(vj.FeatureMode.Basic)
    assert len(pool) == g["features"]
    n = npos + nneg
    labels = np.array([1] * npos + [-1] * nneg, np.int8)
    d_p = torch.from_numpy(p).cuda()
    sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
    inv = torch.empty(n, dtype=torch.float32, device="cuda")
    vj._capi.call("vj_integral_batch", d_p.data_ptr(), 24, 24, 24, n, sumT.data_ptr(), None, inv.data_ptr(), None)
    w0 = np.where(labels > 0, np.float32(0.5) / np.float32(npos), np.float32(0.5) / np.float32(nneg))
    w = torch.from_numpy(w0.astype(np.float32)).cuda()
    lab = torch.from_numpy(labels).cuda()
    t = vj.AdaBoostTrainer((24, 24), n)
    assert t.setFeaturePool(pool) == 0
    assert t.bindTrainingSet(dict(nSamples=n, d_sumT=sumT, d_invNorm=inv), lab, None, w) == 0
    assert t.prepareStage() == 0
    used = torch.zeros(len(pool), dtype=torch.uint8, device="cuda")
    best = torch.zeros(4, dtype=torch.int32, device="cuda")
    strong = torch.zeros(n, dtype=torch.float32, device="cuda")
    weak = torch.zeros(7, dtype=torch.int32, device="cuda")
    calib = torch.zeros(8, dtype=torch.int32, device="cuda")
    same_weights = 0
    for want in g["picks"]:
        r = want["round"]
        assert t.bestWeak(used, best) == 0
        b = best.cpu().numpy().view(vj.TILE_BEST)[0]
        got = (int(b["featureIdx"]), f32bits(b["bestErr"]), f32bits(b["bestTheta"]), int(b["bestParity"]))
        assert got == (want["featureIdx"], want["err_bits"], want["theta_bits"], want["parity"]), r
        assert t.applyBestWeak(best, strong, used, weak) == 0
        assert t.calibrateStage(strong, npos, g["min_hit_rate"], g["max_false_alarm"], nneg, calib) == 0
        c = calib.cpu().numpy().view(vj.STAGE_CALIB)[0]
        wc = want["calib"]
        assert (f32bits(c["cutVal"]), f32bits(c["stageThreshold"]), int(c["strictGt"]), int(c["posPass"]),
                int(c["negSurvive"]), int(c["satisfied"])) == (
            wc["cutVal_bits"], wc["stageThreshold_bits"], wc["strictGt"], wc["posPass"], wc["negSurvive"],
            wc["satisfied"]), r
        assert sha(strong.cpu().numpy()) == want["strong_sha256"], r
        same_weights += sha(w.cpu().numpy()) == want["weights_sha256"]
    wd = w.cpu().numpy().view(np.int32).astype(np.int64)
    wf = final["weights"].view(np.int32).astype(np.int64)
    assert np.abs(wd - wf).max() <= 1
    assert np.array_equal(strong.cpu().numpy().view(np.uint32), final["strong"].view(np.uint32))
    print(f"weights bit-equal to the oracle's after {same_weights} of {len(g['picks'])} rounds")
