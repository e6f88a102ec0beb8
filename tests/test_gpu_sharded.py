"""Feature-range sharding of the device stump search.  Each rank's trainer
sorts and searches only its range of the pool (setSearchRange, one feature
tile of the reference's round loop, src/main.cu:2013-2053); the ranks'
16-byte candidates are gathered into one device array and reduced there by
vj_reduce_tile_best (the reference's ReduceTileBestCandidatesKernel,
src/main.cu:991-1028), and every rank applies the global pick with
vj_round_update.  The picks and final weights equal the single-trainer search
round after round, including a tie across the two ranges (the best feature
copied into the other range), which goes to the lower featureIdx.

Two forms: both ranges in one process on the one GPU (the device arrays the
NCCL all-gather would fill), and two processes with a gloo group, whose
exchange (sharded.exchange_best_device) moves the 16 bytes through the host,
so no kernel waits on the other rank."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
ROUNDS = 4


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _Rank:
    """One rank's trainer over the shared training set, searching [b, e)."""

    def __init__(self, torch, vj, feats, rng_range=None):
        npos = nneg = 300
        p = vj.synth_patches(23, npos, nneg)
        labels = np.array([1] * npos + [-1] * nneg, np.int8)
        n = len(labels)
        self.d_p = torch.from_numpy(p.reshape(-1)).cuda()
        self.sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
        self.inv = torch.empty(n, dtype=torch.float32, device="cuda")
        vj._capi.call("vj_integral_batch", self.d_p.data_ptr(), 24, 24, 24, n, self.sumT.data_ptr(), None,
                      self.inv.data_ptr(), None)
        self.lab = torch.from_numpy(labels).cuda()
        self.w = torch.full((n,), 1.0 / n, dtype=torch.float32, device="cuda")
        self.t = vj.AdaBoostTrainer((24, 24), n)
        assert self.t.setFeaturePool(feats.view(vj.HAAR_FEATURE)) == 0
        if rng_range is not None:
            assert self.t.setSearchRange(rng_range[0], rng_range[1] - rng_range[0]) == 0
        assert self.t.bindTrainingSet(dict(nSamples=n, d_sumT=self.sumT, d_invNorm=self.inv), self.lab, None,
                                      self.w) == 0
        assert self.t.prepareStage() == 0
        self.local = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.best = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.strong = torch.zeros(n, dtype=torch.float32, device="cuda")
        self.used = torch.zeros(len(feats), dtype=torch.uint8, device="cuda")


def _pick(vj, best):
    b = best.cpu().numpy().view(vj.TILE_BEST)[0]
    return (int(b["featureIdx"]), np.float32(b["bestErr"]).tobytes(), np.float32(b["bestTheta"]).tobytes(),
            int(b["bestParity"]))


def _single(torch, vj, feats, rounds=ROUNDS):
    r = _Rank(torch, vj, feats)
    picks = []
    for _ in range(rounds):
        assert r.t.bestWeak(r.used, r.best) == 0
        picks.append(_pick(vj, r.best))
        assert r.t.applyBestWeak(r.best, r.strong, r.used) == 0
    return picks, r.w.cpu().numpy().tobytes()


def _tied_pool(torch, vj, basic_pool):
    feats = np.ascontiguousarray(basic_pool[:40000]).copy()
    first, _ = _single(torch, vj, feats, rounds=1)
    f = first[0][0]
    dup = len(feats) - 1 if f < len(feats) // 2 else 0
    feats[dup] = feats[f]  # the same stump in both ranges: a cross-rank tie
    return feats, min(f, dup)


def test_ranges_reduced_on_device_equal_single_trainer(cuda, vj, basic_pool):
    torch = cuda
    from cs677s26_gb300 import sharded
    feats, lower = _tied_pool(torch, vj, basic_pool)
    want, w_want = _single(torch, vj, feats)
    assert want[0][0] == lower
    world = 2
    ranks = [_Rank(torch, vj, feats, sharded.feature_range(len(feats), k, world)) for k in range(world)]
    gathered = torch.zeros(4 * world, dtype=torch.int32, device="cuda")
    for r_ in range(ROUNDS):
        for k, r in enumerate(ranks):
            assert r.t.bestWeak(r.used, r.local) == 0
            gathered[4 * k:4 * k + 4].copy_(r.local)  # what the all-gather leaves in every rank's array
        for r in ranks:
            vj._capi.call("vj_reduce_tile_best", gathered.data_ptr(), world, r.best.data_ptr(), None)
            assert _pick(vj, r.best) == want[r_]
            assert r.t.applyBestWeak(r.best, r.strong, r.used) == 0
    for r in ranks:
        assert r.w.cpu().numpy().tobytes() == w_want


def test_reduce_tile_best_rule(cuda, vj):
    """Lower error first, -0.0 ties +0.0, then the lower featureIdx; records
    without a split (featureIdx -1, infinite error) win only when alone."""
    torch = cuda
    recs = np.zeros(5, dtype=vj.TILE_BEST)
    recs["bestErr"] = [0.25, 0.0, -0.0, np.inf, 0.125]
    recs["featureIdx"] = [3, 900, 700, -1, 5]
    recs["bestTheta"] = [1, 2, 3, 4, 5]
    out = torch.zeros(4, dtype=torch.int32, device="cuda")
    for sub, want in [(recs, 700), (recs[[0, 4]], 5), (recs[[3, 0]], 3), (recs[[3, 3]], -1), (recs[[1]], 900)]:
        d = torch.from_numpy(np.ascontiguousarray(sub).view(np.int32).copy()).cuda()
        vj._capi.call("vj_reduce_tile_best", d.data_ptr(), len(sub), out.data_ptr(), None)
        assert int(out.cpu().numpy().view(vj.TILE_BEST)[0]["featureIdx"]) == want


def _rank_main(rank, world, port, feats, results):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import cs677s26_gb300 as vj
    from cs677s26_gb300 import sharded

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = _Rank(torch, vj, feats, sharded.feature_range(len(feats), rank, world))
    picks = []
    for _ in range(ROUNDS):
        assert r.t.bestWeak(r.used, r.local) == 0
        sharded.exchange_best_device(r.local, r.best)
        picks.append(_pick(vj, r.best))
        assert r.t.applyBestWeak(r.best, r.strong, r.used) == 0
    torch.cuda.synchronize()
    results[rank] = (picks, r.w.cpu().numpy().tobytes())
    dist.destroy_process_group()


def test_two_ranks_on_device_equal_single_process(cuda, vj, basic_pool):
    import torch.multiprocessing as mp

    feats, _ = _tied_pool(cuda, vj, basic_pool)
    want, w_want = _single(cuda, vj, feats)
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, feats, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(600)
        assert p.exitcode == 0
    for r in range(2):
        picks, w = results[r]
        assert picks == want and w == w_want
