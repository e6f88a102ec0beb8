"""Generates tests/golden/stage_step_picks.json: the 50 stump picks of the full
stage training step (10,000 face + 10,000 texture patches of 24x24 from seed
1, all 162,336 Basic features, uniform initial weights 0.5/10,000, 50
boosting rounds with the FP64 round update and the stage calibration after
every round).

Each round's pick is the oracle's restatement of runCpuWeakSearch
(main.cu:587-682) over the features not yet used, in its stage-resident form
(oracle.SortedPool: every feature sorted once, since the responses do not
change within a stage); the oracle itself is pinned to the reference's CPU
functions by golden.json.  Where the reference's CPU functions are built
(oracle/_ref/libvjref.so), the rounds named by --ref-rounds are also searched
by the reference's own runCpuWeakSearch over the same weights, split over
threads by feature range, and must agree bit for bit.

Per round the fixture stores featureIdx, the FP32 error, theta (as float
bits), parity, the split position, the FP64 error of the same split, the FP32
gap to the runner-up feature, the stage calibration's fields, and sha256 of
the weights and strong scores after the update; plus the final weights and
strong scores in stage_step_final.npz.

    python tests/golden/make_stage_step_picks.py [--threads 8] [--ref-rounds 0,1,2,49|all|none]

Needs about 20 GB of host memory and a few minutes on 8 cores (plus about
half a minute per reference round).
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import json
import sys
import threading
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402

NPOS = NNEG = 10000
ROUNDS = 50
SEED = 1
MIN_HIT, MAX_FA = 0.99, 0.4


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def bits(x) -> int:
    return int(np.array([x], dtype=np.float32).view(np.uint32)[0])


def ref_round(R, pool, patches, labels, w, used, threads):
    """The reference's runCpuWeakSearch over the unused features, split into
    `threads` contiguous feature ranges (one call each, in parallel); the
    ranges' winners combine by the reference's cross-feature rule (lower
    FP32 error, then lower featureIdx)."""
    keep = np.nonzero(used == 0)[0]
    parts = np.array_split(keep, threads)
    out = [None] * len(parts)

    def run(k):
        idx = parts[k]
        feats = np.ascontiguousarray(pool[idx])
        a, e, t, p = C.c_int(), C.c_float(), C.c_float(), C.c_int()
        R.ref_weak_search(feats.ctypes.data, len(feats), patches.ctypes.data, len(labels), labels.ctypes.data, None,
                          w.ctypes.data, C.byref(a), C.byref(e), C.byref(t), C.byref(p))
        if a.value >= 0:
            out[k] = (np.float32(e.value), int(idx[a.value]), bits(t.value), p.value)

    ths = [threading.Thread(target=run, args=(k,)) for k in range(len(parts)) if len(parts[k])]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    e, f, t, p = min(x for x in out if x is not None)
    return {"featureIdx": f, "err_bits": bits(e), "theta_bits": t, "parity": p}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--ref-rounds", default="0,1,2,3,24,49")
    args = ap.parse_args()
    t0 = time.time()
    patches = O.synth_patches(SEED, NPOS, NNEG)
    n = len(patches)
    labels = np.array([1] * NPOS + [-1] * NNEG, np.int8)
    pool = O.feature_pool(0)
    sums, inv = O.train_integrals(patches)
    sp = O.SortedPool(pool, sums, inv, threads=args.threads)
    print(f"sorted {len(pool)} features x {n} samples in {time.time() - t0:.0f} s", flush=True)

    R = O.ref() if O.ref_available() else None
    if args.ref_rounds == "all":
        ref_rounds = set(range(ROUNDS))
    elif args.ref_rounds == "none" or R is None:
        ref_rounds = set()
    else:
        ref_rounds = {int(x) for x in args.ref_rounds.split(",")}

    w = np.where(labels > 0, np.float32(0.5) / np.float32(NPOS), np.float32(0.5) / np.float32(NNEG)).astype(np.float32)
    strong = np.zeros(n, np.float32)
    used = np.zeros(len(pool), np.uint8)
    rounds = []
    for r in range(ROUNDS):
        b, per = sp.search(labels, w, used=used, threads=args.threads, per_feature=True)
        if b["featureIdx"] < 0:
            raise SystemExit(f"round {r}: no valid split")
        errs = per["err"].copy()
        errs[b["featureIdx"]] = np.inf
        ru = int(np.argmin(errs))
        rec = {"round": r, "featureIdx": b["featureIdx"], "err_bits": bits(b["err"]), "theta_bits": bits(b["theta"]),
               "parity": b["parity"], "split": b["split"], "err_fp64": b["err64"],
               "runner_up_featureIdx": ru, "runner_up_gap_fp32": float(np.float32(errs[ru]) - np.float32(b["err"]))}
        if r in ref_rounds:
            t1 = time.time()
            rr = ref_round(R, pool, patches, labels, w, used, args.threads)
            mine = {k: rec[k] for k in ("featureIdx", "err_bits", "theta_bits", "parity")}
            if rr != mine:
                raise SystemExit(f"round {r}: reference {rr} != oracle {mine}")
            rec["reference_checked"] = True
            print(f"round {r}: reference runCpuWeakSearch agrees ({time.time() - t1:.0f} s)", flush=True)
        O.round_update(pool, b, sums, inv, labels, w, strong)
        used[b["featureIdx"]] = 1
        cal = O.stage_calibrate(strong, NPOS, MIN_HIT, MAX_FA, NNEG)
        rec["calib"] = {"cutVal_bits": bits(cal["cutVal"]), "stageThreshold_bits": bits(cal["stageThreshold"]),
                        "strictGt": cal["strictGt"], "posPass": cal["posPass"], "negSurvive": cal["negSurvive"],
                        "satisfied": cal["satisfied"]}
        rec["weights_sha256"] = sha(w)
        rec["strong_sha256"] = sha(strong)
        rounds.append(rec)
        print(f"round {r}: feature {rec['featureIdx']} err {b['err']:.7g} (fp64 {b['err64']:.7g}) "
              f"runner-up gap {rec['runner_up_gap_fp32']:.3g}", flush=True)
    sp.close()
    out = {"about": "full stage training step (10,000 + 10,000 patches, 162,336 Basic features, 50 rounds) "
                    "picks of the oracle's runCpuWeakSearch restatement; see make_stage_step_picks.py",
           "seed": SEED, "npos": NPOS, "nneg": NNEG, "features": int(len(pool)), "rounds": ROUNDS,
           "min_hit_rate": MIN_HIT, "max_false_alarm": MAX_FA, "patches_sha256": sha(patches),
           "reference_rounds": sorted(ref_rounds), "seconds": round(time.time() - t0, 1), "picks": rounds}
    (HERE / "stage_step_picks.json").write_text(json.dumps(out, indent=1) + "\n")
    np.savez_compressed(HERE / "stage_step_final.npz", weights=w, strong=strong)
    print(f"wrote stage_step_picks.json and stage_step_final.npz in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
