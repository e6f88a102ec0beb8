"""Feature-range sharding of the best-weak search over ranks (one GPU each).

The stump search is independent per feature, so ranks split the pool into
contiguous feature ranges, the reference's feature tiles
(src/main.cu:2013-2053).  Each rank sorts and searches only its range
(AdaBoostTrainer.setSearchRange: its resident orders and sweeps cover that
range alone) and finds the range's best stump with the reference's exact pick
rule.  One exchange per round - an all-gather of one 16-byte candidate
(vj_tile_best) per rank into a device array, reduced on the device by
vj_reduce_tile_best, the reference's ReduceTileBestCandidatesKernel
(src/main.cu:991-1028: lower FP32 error, then lower featureIdx) - gives every
rank the global pick, and every rank applies the same round update, so the
weights stay identical across ranks without further traffic.

This is the only collective of the training path; detection and serving
shard by image with no collective at all.

Host-side helpers (pick_global, exchange_best) apply the same rule to plain
records, for ranks that search with the CPU oracle.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

# one record: FP32 error, featureIdx, theta, parity (FP32 values kept bit for bit)
RECORD = np.dtype([("err", "<f4"), ("featureIdx", "<i4"), ("theta", "<f4"), ("parity", "<i4")])


def feature_range(n_features: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of the pool owned by `rank` (sizes differ by at most 1)."""
    if not (0 <= rank < world):
        raise ValueError("rank outside the world")
    return n_features * rank // world, n_features * (rank + 1) // world


def _key(rec) -> tuple[float, int]:
    """The reference's cross-candidate order: FP32 error compared as a float
    (so -0.0 and +0.0 tie), then featureIdx; records without a valid split
    (featureIdx < 0, or an infinite or NaN error) come last."""
    e = float(np.float32(rec["err"]))
    if not np.isfinite(e) or rec["featureIdx"] < 0:
        return (float("inf"), 2**31)
    return (e, int(rec["featureIdx"]))


def pick_global(records: Sequence) -> np.void:
    """The global pick among the ranks' local picks."""
    arr = np.asarray(records, dtype=RECORD).reshape(-1)
    return arr[min(range(len(arr)), key=lambda i: _key(arr[i]))]


def exchange_best(local, group=None) -> np.void:
    """All-gathers every rank's local pick on the host (any backend) and
    returns the global one; `local` has the RECORD fields, featureIdx
    already global."""
    import torch
    import torch.distributed as dist

    rec = np.zeros(1, dtype=RECORD)
    for k in RECORD.names:
        rec[k] = local[k]
    words = torch.from_numpy(rec.view(np.int32).copy())
    world = dist.get_world_size(group)
    out = [torch.zeros_like(words) for _ in range(world)]
    dist.all_gather(out, words, group=group)
    allrec = np.concatenate([o.numpy() for o in out]).view(RECORD)
    return pick_global(allrec)


def exchange_best_device(local, out, gathered=None, group=None, stream=None):
    """The round's exchange on the device.  `local` is this rank's candidate
    (a CUDA int32 tensor of 4 words: vj_tile_best) and `out` receives the
    global pick (same shape).  With NCCL the candidates are all-gathered into
    a device array with no host synchronisation; other backends (gloo) move
    the 16 bytes through the host.  The array is then reduced on the device by
    vj_reduce_tile_best.  `gathered` may hold a reusable int32 CUDA buffer of
    4 * world words."""
    import torch
    import torch.distributed as dist

    from . import _capi

    world = dist.get_world_size(group)
    if gathered is None:
        gathered = torch.empty(4 * world, dtype=torch.int32, device=local.device)
    if dist.get_backend(group) == "nccl":
        dist.all_gather_into_tensor(gathered, local, group=group)
    else:
        parts = [torch.zeros(4, dtype=torch.int32) for _ in range(world)]
        dist.all_gather(parts, local.cpu(), group=group)
        gathered.copy_(torch.cat(parts))
    _capi.call("vj_reduce_tile_best", gathered.data_ptr(), world, out.data_ptr(),
               None if stream is None else int(stream))
    return out


def range_used_mask(n_features: int, rank: int, world: int) -> np.ndarray:
    """A used-feature mask that keeps a full-pool search to this rank's range
    (features marked used are skipped), for ranks searching with the oracle."""
    b, e = feature_range(n_features, rank, world)
    m = np.ones(n_features, np.uint8)
    m[b:e] = 0
    return m
