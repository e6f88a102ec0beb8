"""Feature-range sharding of the stump search over two ranks (gloo, CPU): the
picks after the one-record exchange equal the single-process pick of the
oracle's restatement of runCpuWeakSearch (src/main.cu:587-682), round after
round with the replicated update, and ties across ranks go to the lower
featureIdx as in the reference's cross-feature rule."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(n_pos=120, n_neg=120, n_feat=3000):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import cs677s26_gb300 as V
    import oracle as O
    pool = np.ascontiguousarray(V.feature_pool(V.FeatureMode.Basic)[:n_feat]).view(O.FEATURE)
    pool = pool.copy()
    patches = V.synth_patches(5, n_pos, n_neg)
    labels = np.array([1] * n_pos + [-1] * n_neg, np.int8)
    w = np.full(len(labels), np.float32(1.0) / np.float32(len(labels)), np.float32)
    # the best feature copied into the other rank's half: a cross-rank tie
    sums, inv = O.train_integrals(patches)
    f = O.weak_search(pool, sums, inv, labels, w, threads=2)["featureIdx"]
    dup = n_feat - 1 if f < n_feat // 2 else 0
    pool[dup] = pool[f]
    return O, pool, patches, labels, w, (f, dup)


def _rank_main(rank, world, port, results):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    from cs677s26_gb300 import sharded
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    O, pool, patches, labels, w, _ = _case()
    sums, inv = O.train_integrals(patches)
    strong = np.zeros(len(labels), np.float32)
    used = np.zeros(len(pool), np.uint8)
    picks = []
    for _ in range(3):
        mask = np.maximum(used, sharded.range_used_mask(len(pool), rank, world))
        loc = O.weak_search(pool, sums, inv, labels, w, used=mask, threads=2)
        rec = dict(err=loc["err"], featureIdx=loc["featureIdx"], theta=loc["theta"], parity=loc["parity"])
        g = sharded.exchange_best(rec)
        best = dict(featureIdx=int(g["featureIdx"]), err=float(g["err"]), theta=float(g["theta"]),
                    parity=int(g["parity"]))
        picks.append((best["featureIdx"], best["err"], best["theta"], best["parity"]))
        O.round_update(pool, best, sums, inv, labels, w, strong)  # replicated on every rank
        used[best["featureIdx"]] = 1
    results[rank] = picks
    dist.destroy_process_group()


def test_feature_ranges_cover_the_pool():
    sys.path.insert(0, str(ROOT))
    from cs677s26_gb300 import sharded
    for n, world in [(162336, 2), (162336, 8), (7, 3), (3, 4)]:
        rs = [sharded.feature_range(n, r, world) for r in range(world)]
        assert rs[0][0] == 0 and rs[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
        assert max(e - b for b, e in rs) - min(e - b for b, e in rs) <= 1


def test_pick_global_rule():
    sys.path.insert(0, str(ROOT))
    from cs677s26_gb300 import sharded
    recs = [(0.25, 90, 1.0, 1), (0.125, 500, 2.0, -1), (0.125, 40, 3.0, 1), (float("inf"), 1, 0.0, 1),
            (-0.0, 600, 0.0, 1), (0.0, 700, 0.0, 1)]
    g = sharded.pick_global(recs)
    assert g["featureIdx"] == 600  # below every positive error; -0.0 and +0.0 tie, the lower index wins
    g = sharded.pick_global([(0.0, 600, 0.0, 1), (-0.0, 700, 0.0, 1)])
    assert g["featureIdx"] == 600  # as in the reference's float comparison, not the sign bit
    g = sharded.pick_global(recs[:4])
    assert g["featureIdx"] == 40 and g["theta"] == np.float32(3.0)
    g = sharded.pick_global([(float("inf"), -1, 0.0, 1), (float("inf"), -1, 0.0, 1)])
    assert g["featureIdx"] == -1  # no rank has a valid split


def test_two_ranks_equal_single_process():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    O, pool, patches, labels, w, tie = _case()
    sums, inv = O.train_integrals(patches)
    strong = np.zeros(len(labels), np.float32)
    used = np.zeros(len(pool), np.uint8)
    want = []
    for _ in range(3):
        b = O.weak_search(pool, sums, inv, labels, w, used=used, threads=4)
        want.append((b["featureIdx"], b["err"], b["theta"], b["parity"]))
        O.round_update(pool, b, sums, inv, labels, w, strong)
        used[b["featureIdx"]] = 1
    assert results[0] == results[1] == want
    assert want[0][0] == min(tie)  # the tied pair sits on both ranks; the lower index wins
