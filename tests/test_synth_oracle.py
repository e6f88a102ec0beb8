"""The oracle's own restatement of the synthetic generators (oracle/vj_synth.c)
gives the same bytes as the package's (csrc/synth.cpp): the CPU legs of the
benchmark and the fixture scripts build their inputs from it without loading
the product library.  And the oracle's stage-resident search (SortedPool)
gives the per-call search's picks, pinned by the golden rounds of the
reference's own runCpuWeakSearch."""
import numpy as np
import pytest

from conftest import f32


@pytest.mark.parametrize("seed,npos,nneg", [(1, 300, 300), (677, 50, 70), (31, 160, 160), (9, 0, 5)])
def test_patches(vj, oracle, seed, npos, nneg):
    assert np.array_equal(oracle.synth_patches(seed, npos, nneg), vj.synth_patches(seed, npos, nneg))


@pytest.mark.parametrize("args", [(1, 1920, 1080, 40, 24, 300), (7, 320, 240, 6, 24, 120), (1003, 333, 250, 5, 24, 300),
                                  (5, 97, 61, 1, 24, 61), (2, 24, 24, 3, 24, 24)])
def test_scenes(vj, oracle, args):
    assert np.array_equal(oracle.synth_scene(*args), vj.synth_scene(*args))


@pytest.mark.parametrize("shape", [(12, 400), (38, 6061)])
def test_cascades(vj, oracle, shape):
    a, b = oracle.synth_cascade(2, *shape), vj.synth_cascade(2, *shape)
    assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def test_sorted_pool_rounds_equal_the_reference(oracle, golden, basic_pool):
    g = golden["rounds"]
    p = oracle.synth_patches(g["seed"], g["npos"], g["nneg"])
    labels = np.array([1] * g["npos"] + [-1] * g["nneg"], np.int8)
    feats = np.ascontiguousarray(basic_pool[: g["features"]])
    sums, inv = oracle.train_integrals(p)
    sp = oracle.SortedPool(feats, sums, inv, threads=8)
    w = np.full(len(labels), np.float32(0.5) / np.float32(g["npos"]), np.float32)
    strong = np.zeros(len(labels), np.float32)
    used = np.zeros(len(feats), np.uint8)
    rng = np.random.default_rng(3)
    for r in g["picks"]:
        b = sp.search(labels, w, used=used)
        assert (b["featureIdx"], b["err"], b["theta"], b["parity"]) == (
            r["featureIdx"], f32(r["err_bits"]), f32(r["theta_bits"]), r["parity"])
        # with an active mask too, equal to the per-call search
        act = (rng.random(len(labels)) > 0.3).astype(np.uint8)
        assert sp.search(labels, w, active=act, used=used) == oracle.weak_search(feats, sums, inv, labels, w,
                                                                                 active=act, used=used)
        oracle.round_update(feats, b, sums, inv, labels, w, strong)
        used[b["featureIdx"]] = 1
    sp.close()
