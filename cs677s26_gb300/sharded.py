"""Feature-range sharding of the best-weak search over ranks (one GPU each).

The stump search is independent per feature, so ranks split the pool into
contiguous feature ranges.  Each rank finds its range's best stump with the
reference's exact pick rule (vj_stump_search with the features outside its
range marked used, or a trainer over its range), and one exchange per round -
an all-gather of one (FP32 error, featureIdx, theta, parity) record per rank -
selects the global pick by the reference's cross-feature rule: lower FP32
error, then lower featureIdx (ReduceTileBestCandidatesKernel and
SelectBestInTileKernel's tie-break, src/main.cu:999-1028,
src/boosting_core.cu:87-99).  Every rank then applies the same round update,
so weights stay identical across ranks without further traffic.

This is the only collective of the training path; detection and serving
shard by image with no collective at all.
"""
from __future__ import annotations

import struct
from typing import Sequence

import numpy as np

# one record: FP32 error, featureIdx, theta, parity (FP32 values kept bit for bit)
RECORD = np.dtype([("err", "<f4"), ("featureIdx", "<i4"), ("theta", "<f4"), ("parity", "<i4")])


def feature_range(n_features: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of the pool owned by `rank` (sizes differ by at most 1)."""
    if not (0 <= rank < world):
        raise ValueError("rank outside the world")
    return n_features * rank // world, n_features * (rank + 1) // world


def _key(rec) -> tuple[int, int]:
    """Order of the reference's cross-feature rule: FP32 error (as an ordered
    integer; NaN/inf never win), then featureIdx."""
    e = float(np.float32(rec["err"]))
    if not np.isfinite(e) or rec["featureIdx"] < 0:
        return (2**32, 2**31)
    bits = struct.unpack("<I", struct.pack("<f", e))[0]
    ordered = bits ^ 0x80000000 if bits < 0x80000000 else ~bits & 0xFFFFFFFF  # float order as unsigned
    return (ordered, int(rec["featureIdx"]))


def pick_global(records: Sequence) -> np.void:
    """The global pick among the ranks' local picks."""
    arr = np.asarray(records, dtype=RECORD).reshape(-1)
    return arr[min(range(len(arr)), key=lambda i: _key(arr[i]))]


def exchange_best(local, group=None) -> np.void:
    """All-gathers every rank's local pick (torch.distributed, any backend)
    and returns the global one; `local` has the RECORD fields, featureIdx
    already global."""
    import torch
    import torch.distributed as dist

    rec = np.zeros(1, dtype=RECORD)
    for k in RECORD.names:
        rec[k] = local[k]
    words = torch.from_numpy(rec.view(np.int32).copy())
    if dist.get_backend(group) == "nccl":
        words = words.cuda()
    world = dist.get_world_size(group)
    out = [torch.zeros_like(words) for _ in range(world)]
    dist.all_gather(out, words, group=group)
    allrec = np.concatenate([o.cpu().numpy() for o in out]).view(RECORD)
    return pick_global(allrec)


def range_used_mask(n_features: int, rank: int, world: int) -> np.ndarray:
    """A used-feature mask that keeps a full-pool trainer to this rank's range
    (vj_stump_search skips features marked used)."""
    b, e = feature_range(n_features, rank, world)
    m = np.ones(n_features, np.uint8)
    m[b:e] = 0
    return m
