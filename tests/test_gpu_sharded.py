"""Feature-range sharding of the device stump search: two ranks (processes
with a gloo group) on the one GPU, each running vj_stump_search over its half
of the pool with the other half masked as used, exchange one record per round
(cs677s26_gb300.sharded.exchange_best) and apply the global pick with
vj_round_update.  No kernel waits on the other rank: the exchange is on the
host.  The picks equal the single-process search round after round, including
a tie across the two halves (the best feature copied into the other half),
which goes to the lower featureIdx as in the reference's cross-feature rule
(src/main.cu:999-1028)."""
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


def _train(rank, world, feats, rounds=ROUNDS):
    import torch

    sys.path.insert(0, str(ROOT))
    import cs677s26_gb300 as vj
    from cs677s26_gb300 import sharded

    npos = nneg = 300
    p = vj.synth_patches(23, npos, nneg)
    labels = np.array([1] * npos + [-1] * nneg, np.int8)
    w0 = np.full(len(labels), np.float32(1.0) / np.float32(len(labels)), np.float32)
    n = len(labels)
    d_p = torch.from_numpy(p.reshape(-1)).cuda()
    sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
    inv = torch.empty(n, dtype=torch.float32, device="cuda")
    vj._capi.call("vj_integral_batch", d_p.data_ptr(), 24, 24, 24, n, sumT.data_ptr(), None, inv.data_ptr(), None)
    lab = torch.from_numpy(labels).cuda()
    w = torch.from_numpy(w0).cuda()
    t = vj.AdaBoostTrainer((24, 24), n)
    assert t.setFeaturePool(feats.view(vj.HAAR_FEATURE)) == 0
    assert t.bindTrainingSet(dict(nSamples=n, d_sumT=sumT, d_invNorm=inv), lab, None, w) == 0
    assert t.prepareStage() == 0
    best = torch.zeros(4, dtype=torch.int32, device="cuda")
    strong = torch.zeros(n, dtype=torch.float32, device="cuda")
    used = np.zeros(len(feats), np.uint8)
    picks = []
    for _ in range(rounds):
        mask = np.maximum(used, sharded.range_used_mask(len(feats), rank, world)) if world > 1 else used
        assert t.bestWeak(torch.from_numpy(mask).cuda(), best) == 0
        rec = best.cpu().numpy().view(vj.TILE_BEST)[0]
        loc = dict(err=rec["bestErr"], featureIdx=rec["featureIdx"], theta=rec["bestTheta"],
                   parity=rec["bestParity"])
        g = sharded.exchange_best(loc) if world > 1 else loc
        out = np.zeros(1, dtype=vj.TILE_BEST)
        out["featureIdx"], out["bestErr"] = g["featureIdx"], g["err"]
        out["bestTheta"], out["bestParity"] = g["theta"], g["parity"]
        best.copy_(torch.from_numpy(out.view(np.int32).copy()).cuda())
        assert t.applyBestWeak(best, strong) == 0
        used[int(g["featureIdx"])] = 1
        picks.append((int(g["featureIdx"]), np.float32(g["err"]).tobytes(), np.float32(g["theta"]).tobytes(),
                      int(g["parity"])))
    torch.cuda.synchronize()
    return picks, w.cpu().numpy().tobytes()


def _rank_main(rank, world, port, feats, results):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    results[rank] = _train(rank, world, feats)
    dist.destroy_process_group()


def test_two_ranks_on_device_equal_single_process(cuda, vj, basic_pool):
    import torch.multiprocessing as mp

    feats = np.ascontiguousarray(basic_pool[:40000]).copy()
    first, _ = _train(0, 1, feats, rounds=1)
    f = first[0][0]
    dup = len(feats) - 1 if f < len(feats) // 2 else 0
    feats[dup] = feats[f]  # the same stump on both halves: a cross-rank tie
    want, w_want = _train(0, 1, feats)
    assert want[0][0] == min(f, dup)
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
