"""Benchmark of the Viola-Jones data-parallel path on GB300.

Workload (a "step"): the full stage training step on 10,000 positive and
10,000 negative synthetic 24x24 patches (seed 1): integral images, per-feature
sort of all 162,336 Basic features (kept resident for the stage), then 50
boosting rounds, each = best-weak search (bit-exact picks of the reference's
search) + FP64 AdaBoost update + stage calibration.

value (stump GB/s): 20 bytes per (feature, sample) per round (f32 key write
+ read, sorted (f32 key, u16 index) pair write + read: one materialisation of
the sort-based algorithm) x 162,336 x 20,000 x 50 / step time.

The same line carries, under "detect", the detection workloads: plain
multiscale detect of a 1920x1080 scene, batched detect of 256 scenes of
uneven sizes, and the serving loop (Poisson arrivals, continuous batching,
16 GiB HBM budget) against plain per-image detect on the same trace, with
images/s and p50/p99/p999 latency; plus a CPU baseline of each.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun (N > 1) the ranks split the
feature pool into contiguous ranges: each sorts and searches its own range,
and every round the ranks all-gather their 16-byte candidates over NCCL into
a device array, reduce it on the device and apply the same round update (the
whole job is one stage step: scaling "strong").  Detection and serving run on
rank 0 only (they shard by image, replicas only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NPOS = NNEG = 10000
ROUNDS = 50
SEED = 1
BYTES_PER_ELEM_ROUND = 20  # algorithmic model of the stump search
# The headline metric of this path; `value` is its stump GB/s part (the stage
# training step), the served images/s and latencies are under "detect".
METRIC = "served images/s + p50/p99 ms vs plain detect at equal dets; stump GB/s"
DTYPE = "f32 (int32 responses, FP64 renorm)"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def sharded_range(F, rank, world):
    return (F * rank // world, F * (rank + 1) // world)


def workload_config(F, n, world):
    """The `config` of both arms' JSON lines."""
    c = {"workload": "full stage training step: 10,000+10,000 24x24 patches (seed 1), "
                     "162,336 Basic features, 50 boosting rounds",
         "features": F, "samples": n, "rounds": ROUNDS,
         "parallelism": "one GPU" if world == 1 else f"feature-range shards x{world} (one 16-byte candidate "
                                                     "all-gathered per round)",
         "l2": "per-round working set (sorted orders 6.9 GB) exceeds L2"}
    if F != 162336 or ROUNDS != 50:
        c["workload"] = f"reduced stage step for profiling: {F} features, {ROUNDS} rounds"
    return c


# ----------------------------------------------------------------------------- GPU arm
class Stage:
    """Device-resident stage-training state for one step.  With world > 1 the
    trainer sorts and searches only this rank's feature range, and each round
    exchanges the ranks' 16-byte candidates (NCCL all-gather into a device
    array, reduced on the device) before the replicated round update."""

    def __init__(self, torch, V, patches, pool, rank=0, world=1):
        self.torch, self.V = torch, V
        n = len(patches)
        self.n = n
        self.numPos = NPOS
        self.d_p = torch.from_numpy(patches).cuda()
        self.sumT = torch.empty(625 * n, dtype=torch.int32, device="cuda")
        self.inv = torch.empty(n, dtype=torch.float32, device="cuda")
        labels = np.array([1] * NPOS + [-1] * NNEG, np.int8)
        self.h_labels = labels
        self.lab = torch.from_numpy(labels).cuda()
        self.w = torch.empty(n, dtype=torch.float32, device="cuda")
        self.w0 = torch.from_numpy(np.where(labels > 0, np.float32(0.5) / np.float32(NPOS),
                                            np.float32(0.5) / np.float32(NNEG)).astype(np.float32)).cuda()
        self.strong = torch.zeros(n, dtype=torch.float32, device="cuda")
        self.used = torch.zeros(len(pool), dtype=torch.uint8, device="cuda")
        self.best = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.weaks = torch.zeros(ROUNDS * 7, dtype=torch.int32, device="cuda")
        self.calib = torch.zeros(8, dtype=torch.int32, device="cuda")
        self.t = V.AdaBoostTrainer((24, 24), n)
        assert self.t.setFeaturePool(pool) == 0
        self.ii = dict(nSamples=n, d_sumT=self.sumT, d_invNorm=self.inv)
        self.world = world
        if world > 1:
            from cs677s26_gb300 import sharded
            self.sharded = sharded
            b, e = sharded.feature_range(len(pool), rank, world)
            assert self.t.setSearchRange(b, e - b) == 0
            self.local = torch.zeros(4, dtype=torch.int32, device="cuda")
            self.gathered = torch.zeros(4 * world, dtype=torch.int32, device="cuda")

    def step(self, stream=None):
        """One stage step: integrals, resident sort, ROUNDS rounds (no host sync)."""
        V, torch = self.V, self.torch
        V._capi.call("vj_integral_batch", self.d_p.data_ptr(), 24, 24, 24, self.n, self.sumT.data_ptr(), None,
                     self.inv.data_ptr(), stream)
        self.w.copy_(self.w0)
        self.strong.zero_()
        self.used.zero_()
        assert self.t.bindTrainingSet(self.ii, self.lab, None, self.w) == 0
        assert self.t.prepareStage(stream) == 0
        for r in range(ROUNDS):
            if self.world > 1:
                assert self.t.bestWeak(self.used, self.local, stream) == 0
                self.sharded.exchange_best_device(self.local, self.best, self.gathered, stream=stream)
            else:
                assert self.t.bestWeak(self.used, self.best, stream) == 0
            wk = self.weaks[r * 7:(r + 1) * 7]
            assert self.t.applyBestWeak(self.best, self.strong, self.used, wk, stream) == 0
            assert self.t.calibrateStage(self.strong, self.numPos, 0.99, 0.4, NNEG, self.calib, stream) == 0


def stump_responses(feat, sumT, inv):
    """FP32 responses of one upright feature for every sample (exact int box
    sums, one FP32 rounding by invNorm): the statement's own arithmetic."""
    raw = np.zeros(sumT.shape[1], np.int64)
    for r in ("r0", "r1", "r2")[: int(feat["rectCount"])]:
        q = feat[r]
        box = sumT[int(q["p0"])] - sumT[int(q["p1"])] - sumT[int(q["p2"])] + sumT[int(q["p3"])]
        raw += box * np.int64(q["w"])
    return (raw.astype(np.float32) * inv).astype(np.float32)


def oracle_picks(F, n):
    """The oracle's 50 picks of this workload (tests/golden/stage_step_picks.json),
    when the step runs the full configuration."""
    path = ROOT / "tests" / "golden" / "stage_step_picks.json"
    if not path.exists():
        return None
    g = json.loads(path.read_text())
    if g["features"] != F or g["npos"] + g["nneg"] != n or g["rounds"] != ROUNDS:
        return None
    return g["picks"]


def f32bits(x) -> int:
    return int(np.array([x], dtype=np.float32).view(np.uint32)[0])


def round_report(V, st, pool):
    """One extra stage step, untimed, read back round by round: the pick's FP32
    error (the reference's sequential FP32 search arithmetic) beside the FP64
    weighted error of the same stump over that round's weights, the FP32 gap
    from the pick to the runner-up among the exactly replayed candidates (null
    when the pick was the only candidate), and whether the pick (featureIdx,
    FP32 error, theta, parity) equals the oracle's for the same round bit for
    bit (tests/golden/stage_step_picks.json)."""
    want = oracle_picks(len(pool), st.n)
    V._capi.call("vj_integral_batch", st.d_p.data_ptr(), 24, 24, 24, st.n, st.sumT.data_ptr(), None,
                 st.inv.data_ptr(), None)
    st.w.copy_(st.w0)
    st.strong.zero_()
    st.used.zero_()
    assert st.t.bindTrainingSet(st.ii, st.lab, None, st.w) == 0
    assert st.t.prepareStage() == 0
    sumT = st.sumT.cpu().numpy().reshape(625, st.n).astype(np.int64)
    inv = st.inv.cpu().numpy()
    rows = []
    for r in range(ROUNDS):
        w = st.w.cpu().numpy().astype(np.float64)
        assert st.t.bestWeak(st.used, st.best) == 0
        info = st.t.lastRound()
        b = st.best.cpu().numpy().view(V.TILE_BEST)[0]
        f, theta, par = int(b["featureIdx"]), np.float32(b["bestTheta"]), int(b["bestParity"])
        left = stump_responses(pool[f], sumT, inv) < theta
        pred = np.where(left, -1, 1) if par > 0 else np.where(left, 1, -1)
        e64 = float(w[pred != st.h_labels].sum())
        e32 = float(b["bestErr"])
        ru = info["runnerUpErr"]
        row = {"round": r, "featureIdx": f, "err_fp32": e32, "err_fp64": e64, "abs_diff": abs(e32 - e64),
               "runner_up_gap_fp32": (ru - e32) if np.isfinite(ru) else None,
               "candidates": info["candidates"], "window": info["window"], "swept": info["swept"]}
        if want is not None:
            o = want[r]
            row["pick_equals_oracle"] = (f, f32bits(b["bestErr"]), f32bits(b["bestTheta"]), par) == (
                o["featureIdx"], o["err_bits"], o["theta_bits"], o["parity"])
        rows.append(row)
        wk = st.weaks[r * 7:(r + 1) * 7]
        assert st.t.applyBestWeak(st.best, st.strong, st.used, wk) == 0
        assert st.t.calibrateStage(st.strong, st.numPos, 0.99, 0.4, NNEG, st.calib) == 0
    gaps = [x["runner_up_gap_fp32"] for x in rows if x["runner_up_gap_fp32"] is not None]
    eq = [x["pick_equals_oracle"] for x in rows if "pick_equals_oracle" in x]
    return {"rounds": rows, "max_abs_err_diff": max(x["abs_diff"] for x in rows),
            "picks_equal_oracle": f"{sum(eq)}/{len(eq)}" if eq else None,
            "min_runner_up_gap": min(gaps) if gaps else None,
            "rounds_gap_below_diff": sum(1 for x in rows if x["runner_up_gap_fp32"] is not None and
                                         x["runner_up_gap_fp32"] <= x["abs_diff"])}


def profile_read(V, reset=True):
    import ctypes as C
    lib = V.load()
    n = C.c_int()
    lib.vj_profile_read(None, 0, C.byref(n), 0)
    buf = (C.c_char * (64 * max(1, n.value)))()
    lib.vj_profile_read(C.addressof(buf), n.value, C.byref(n), int(reset))
    out = {}
    raw = bytes(buf)
    for i in range(n.value):
        rec = raw[i * 64:(i + 1) * 64]
        name = rec[:48].split(b"\0")[0].decode()
        launches = int.from_bytes(rec[48:56], "little", signed=True)
        ms = float(np.frombuffer(rec[56:64], dtype=np.float64)[0])
        out[name] = (launches, ms)
    return out


def run_gpu(args, rank, world):
    import torch

    import cs677s26_gb300 as V

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pool = V.feature_pool(V.FeatureMode.Basic)[: args.features]
    F = len(pool)
    patches = V.synth_patches(SEED, NPOS, NNEG)
    n = len(patches)
    st = Stage(torch, V, patches, pool, rank, world)
    # warm-up
    for _ in range(args.warmup):
        st.step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    V.load().vj_profile_enable(1)
    profile_read(V, reset=True)
    swept0 = st.t.lastRound()["sweptTotal"] if args.warmup > 0 else 0
    with Clocks(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0.record()
        for _ in range(args.steps):
            st.step()
        t1.record()
        torch.cuda.synchronize()
    V.load().vj_profile_enable(0)
    prof = profile_read(V, reset=True)
    # features the sweeps streamed in the timed steps (the rest were pruned by
    # their error bounds, or used)
    swept_timed = st.t.lastRound()["sweptTotal"] - swept0
    ms = t0.elapsed_time(t1)
    if dist:
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
        if dist:
            dist.barrier()
    ms_step = ms / args.steps
    # the whole job's work: one stage step over the full pool, split over the
    # ranks' feature ranges (strong scaling)
    units = BYTES_PER_ELEM_ROUND * F * n * ROUNDS
    value = units / (ms_step * 1e-3) / 1e9

    # picks of the last step (sanity: deterministic across steps)
    weaks = st.weaks.cpu().numpy().view(V.WEAK)

    # ---- end to end through the C ABI with host buffers: upload the patches,
    # train the step, read the 50 weak classifiers back.
    h_p = torch.from_numpy(patches).pin_memory()
    h_w = torch.empty(ROUNDS * 7, dtype=torch.int32).pin_memory()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    e0.record()
    for _ in range(e2e_steps):
        st.d_p.copy_(h_p, non_blocking=True)
        st.step()
        h_w.copy_(st.weaks, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / e2e_steps
    if dist:
        tt = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_e2e = float(tt.item())
    e2e_value = units / (ms_e2e * 1e-3) / 1e9

    # ---- roofline of the dominant kernel (and of both large kernels)
    peak, peak_kind = peaks()
    ord_stride = (n + 7) & ~7
    gap_stride = (n + 31) // 32
    F_local = len(range(*sharded_range(F, rank, world)))
    sweeps = max(1, prof.get("sweep_kernel", (1, 0.0))[0])
    swept_per_launch = swept_timed / sweeps
    kbytes = {
        # resident sweep: sorted order (2 B) + split bitmask (1/8 B) per
        # feature-sample, for the features a launch streams
        "sweep_kernel": swept_per_launch * (ord_stride * 2 + gap_stride * 4),
        # eval+sort: reads the L2-resident integrals, writes order + bitmask
        "eval_sort_kernel": F_local * (ord_stride * 2 + gap_stride * 4) + 625 * n * 4,
    }
    units_per_launch = {"sweep_kernel": swept_per_launch * n, "eval_sort_kernel": F_local * n}
    # DRAM bytes (read + write) per feature-sample of one launch, from ncu's
    # dram__bytes counters on the 16,384-feature x 20,000-sample case, scaled
    # to this launch's size.
    traffic_per_unit = {"sweep_kernel": (713.343488e6 + 3.387648e6) / (16384 * 20000),
                        "eval_sort_kernel": (227.704576e6 + 671.324416e6) / (16384 * 20000)}
    notes = {"sweep_kernel": "streams the resident orders once per round; HBM is its roofline",
             "eval_sort_kernel": "once per stage; an on-chip radix sort bound by the shared-memory pipe "
                                 "(per-thread digit counters, random key gathers and index scatters), its "
                                 "HBM fraction is informational"}

    # The sort is bound by the shared-memory pipe, not by HBM: its wavefronts per
    # feature-sample from ncu's l1tex__data_pipe_lsu_wavefronts_mem_shared.sum on
    # the same 16,384 x 20,000 case, against one wavefront per cycle per SM at the
    # SM clock sampled during the timed steps (a nominal figure, not a measured peak).
    smem_wavefronts_per_unit = {"eval_sort_kernel": 1195117053 / (16384 * 20000)}
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count

    def roofline_of(name):
        launches, total = prof[name]
        avg_ms = total / max(1, launches)
        tpu = traffic_per_unit.get(name)
        r = {"kernel": name, "bound": "hbm", "unit": "GB/s", "peak": peak, "peak_kind": peak_kind,
             "avg_launch_ms": avg_ms, "launches": launches, "share_of_step": total / ms if ms else None,
             "traffic": tpu * units_per_launch[name] if tpu else None,
             "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum at 16,384 features x 20,000 "
                               "samples, scaled by features x samples" if tpu else None}
        if name in kbytes:
            ach = kbytes[name] / (avg_ms * 1e-3) / 1e9
            r.update({"achieved": ach, "frac": ach / peak, "algorithmic_bytes_per_launch": kbytes[name]})
        if name in notes:
            r["note"] = notes[name]
        if name in smem_wavefronts_per_unit and avg_ms > 0:
            ach = smem_wavefronts_per_unit[name] * units_per_launch[name] / (avg_ms * 1e-3)
            pk = sms * sm_mhz * 1e6
            r["onchip"] = {"bound": "shared-memory pipe", "unit": "wavefronts/s", "achieved": ach, "peak": pk,
                           "peak_kind": "nominal: 1 wavefront per cycle per SM at the sampled SM clock",
                           "frac": ach / pk,
                           "source": "ncu l1tex__data_pipe_lsu_wavefronts_mem_shared.sum at 16,384 features x "
                                     "20,000 samples, scaled by features x samples"}
        return r

    dom = max(prof.items(), key=lambda kv: kv[1][1])[0] if prof else None
    roof = roofline_of(dom) if dom else None
    rooflines = {k: roofline_of(k) for k in ("sweep_kernel", "eval_sort_kernel") if k in prof}
    gpu_launches = sum(v[0] for v in prof.values())

    result = {
        "metric": METRIC, "value": value, "unit": "GB/s",
        "value_is": "stump GB/s of the stage training step by the 20 B per feature-sample per round model (a "
                    "per-round sort materialised in HBM); an algorithmic throughput that exceeds the HBM peak by "
                    "design, since the sort runs once per stage and pruned features are not streamed; the "
                    "rooflines below measure each kernel against the bytes it moves",
        "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": DTYPE, "data": "synthetic",
        "config": workload_config(F, n, world),
        "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": int(patches.nbytes),
                "d2h_bytes_per_step": int(ROUNDS * 28)},
        "gpu_launches": gpu_launches, "roofline": roof, "rooflines": rooflines,
        "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in sorted(prof.items())},
        "ms_per_round": ms_step / ROUNDS,
        "sweep_pruning": {"features_streamed_per_round": swept_per_launch, "features": F_local,
                          "streamed_fraction": swept_per_launch / F_local if F_local else None,
                          "note": "from the second round of a stage, features whose error bound cannot reach the "
                                  "candidate window are not streamed; picks are unchanged"},
        "clocks": clocks,
        "picks_head": [int(x) for x in weaks["featureIdx"][:5]],
    }
    if rank == 0 and world == 1:
        result["round_report"] = round_report(V, st, pool)
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline()
    if dist:
        dist.destroy_process_group()
        dist = None
    if rank == 0 and not args.no_detect:
        det = run_detect(V, torch, quick=args.quick_detect)
        det["workloads"] = {
            "plain_1080p": "one 1920x1080 synthetic scene (1/f texture, 40 pasted faces 24-300 px), "
                           "scaleFactor 1.25, minNeighbors 4, minObjectSize 24, 38-stage / 6,061-stump cascade; "
                           "host image in, grouped detections out, per call",
            "batch_256": "256 synthetic scenes, sizes log-uniform 320x240..3840x2160 (425.7 MP), same cascade; "
                         "pinned host images in, grouped detections out; one persistent launch per batch",
            "serving": "Poisson arrivals at 200, 400, 500, 600, 1000 and 2000 req/s of requests drawn from the same "
                       "256 scenes, "
                       "the same trace for both servers; 16 GiB HBM budget each; plain = one image per launch "
                       "(maxBatchImages 1, one worker); batched = continuous batching, 2 workers whose kernels "
                       "each fill the GPU and take turns, up to 256 images and 32 MP per launch"}
        result["detect"] = det
    return result


# ----------------------------------------------------------------------------- detection and serving
BATCH_SCENES = 256
BATCH_PIXELS = 32_000_000  # serving batch cap: about 30 ms of device work, well past what fills the GPU


def detect_inputs(V):
    """The synthetic detection workloads: the 38-stage / 6,061-stump cascade,
    one 1920x1080 scene with 40 pasted faces (plain detect), and 256 scenes of
    log-uniform sizes from 320x240 to 3840x2160 with 5 faces each (batched
    detect and serving).  Scenes are generated on all host threads."""
    from concurrent.futures import ThreadPoolExecutor
    pool = V.feature_pool(V.FeatureMode.Basic)
    st, sg = V.synth_cascade(2)
    rng = np.random.default_rng(3)
    sizes = []
    for _ in range(BATCH_SCENES):
        t = rng.random()
        sizes.append((int(round(320 * 12 ** t)), int(round(240 * 9 ** t))))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        scenes = list(ex.map(lambda a: V.synth_scene(1000 + a[0], a[1][0], a[1][1], 5, 24, 300), enumerate(sizes)))
    scene1080 = V.synth_scene(1, 1920, 1080, 40, 24, 300)
    return pool, st, sg, scene1080, scenes


def serve_trace(srv, scenes, rate, n, seed):
    """Poisson arrivals at `rate` req/s of n requests drawn from `scenes`;
    returns the server's statistics and the results in request order."""
    arr = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, n))
    picks = np.random.default_rng(seed + 1).integers(0, len(scenes), n)
    tickets = [None] * n
    res = [None] * n

    def waiter():
        for i in range(n):
            while tickets[i] is None:
                time.sleep(0.0002)
            _, res[i] = srv.wait(tickets[i])

    th = threading.Thread(target=waiter)
    th.start()
    srv.resetStats()
    t0 = time.perf_counter()
    for i in range(n):
        dl = t0 + arr[i] - time.perf_counter()
        if dl > 0:
            time.sleep(dl)
        tickets[i] = srv.submit(scenes[picks[i]])
    th.join()
    return srv.stats(), res, picks


def run_detect(V, torch, quick=False):
    pool, st, sg, scene1080, scenes = detect_inputs(V)
    f, s, g = pool.view(V.HAAR_FEATURE), st.view(V.STUMP4), sg.view(V.STAGE)
    e = V.FaceVisionEngine((24, 24), 1, 3840, 2160, False, 200000)
    assert e.setCascadeModel(f, s, g) == 0
    out = {}
    # ---- plain multiscale detect of one 1920x1080 image (host image in, grouped detections out)
    for _ in range(3):
        e.detectMultiScale(scene1080, 1920, 1080, 1920)
    reps = 10
    t = time.perf_counter()
    for _ in range(reps):
        st_, grp = e.detectMultiScale(scene1080, 1920, 1080, 1920)
    ms = (time.perf_counter() - t) / reps * 1e3
    k = e.lastStats()
    out["plain_1080p"] = {"images_per_s": 1e3 / ms, "ms_per_image": ms, "gpu_ms": k["gpuMs"],
                          "host_ms": k["hostMs"], "phase_ms": k["phaseMs"], "raw_detections": k["rawDetections"],
                          "grouped_detections": int(len(grp)), "windows": k["windows"],
                          "stump_evals": k["stumpEvals"], "stumps_per_s_gpu": k["stumpEvals"] / (k["gpuMs"] * 1e-3)}
    # ---- batched detect of 256 scenes
    s_, cfg, tune_ms = e.autotune(scenes[:32], repeats=1)
    pinned = []
    for sc in scenes:
        tp = torch.from_numpy(sc).pin_memory()
        pinned.append(tp.numpy())
    e.detectBatch(pinned, capPerImage=4096)
    times = []
    for _ in range(2 if quick else 3):
        t = time.perf_counter()
        s_, batch = e.detectBatch(pinned, capPerImage=4096)
        times.append(time.perf_counter() - t)
    kb = e.lastStats()
    bt = statistics.median(times)
    dev = [torch.from_numpy(sc).cuda() for sc in scenes]
    e.detectBatch(dev, capPerImage=4096)
    t = time.perf_counter()
    e.detectBatch(dev, capPerImage=4096)
    bt_dev = time.perf_counter() - t
    del dev
    # plain per-image detect over the same scenes, and the identity check
    t = time.perf_counter()
    same = True
    for i, sc in enumerate(pinned):
        s_, one = e.detectMultiScale(sc, sc.shape[1], sc.shape[0], sc.shape[1])
        same = same and one.tobytes() == batch[i].tobytes()
    pt = time.perf_counter() - t
    px = sum(sc.size for sc in scenes)
    out["batch_256"] = {"images_per_s": len(scenes) / bt, "s_per_batch": bt, "gpu_ms": kb["gpuMs"],
                        "host_ms": kb["hostMs"], "phase_ms": kb["phaseMs"],
                        "images_per_s_device_images": len(scenes) / bt_dev,
                        "megapixels": px / 1e6, "pyramid_pixels": kb["pyramidPixels"], "windows": kb["windows"],
                        "stump_evals": kb["stumpEvals"], "stumps_per_s_gpu": kb["stumpEvals"] / (kb["gpuMs"] * 1e-3),
                        "raw_detections": kb["rawDetections"], "autotuned_config": cfg, "autotune_best_ms_32": tune_ms,
                        "plain_images_per_s_same_scenes": len(scenes) / pt,
                        "batch_over_plain": pt / bt, "identical_to_plain_per_image": bool(same)}
    e = None
    # ---- serving: Poisson arrivals of the same scenes at each rate, continuous
    # batching (2 workers, every kernel on the whole GPU, taking turns) against
    # plain per-image detect (one image per launch), same trace, same results
    serving = {"hbm_budget_gb": (16 << 30) / 1e9, "workers": 2, "max_batch_pixels": BATCH_PIXELS}
    # 400-600 req/s lie between the two servers' capacities (plain about 440,
    # batched about 645 images/s on these scenes): there batching keeps up and
    # plain per-image serving does not
    rates = [200] if quick else [200, 400, 500, 600, 1000, 2000]
    plain = V.DetectServer(f, s, g, workers=1, maxBatchImages=1, hbmBudgetBytes=16 << 30)
    batched = V.DetectServer(f, s, g, workers=2, maxBatchImages=256, maxBatchPixels=BATCH_PIXELS,
                             hbmBudgetBytes=16 << 30, tileRows=cfg["tileRows"], tileStumps=cfg["tileStumps"])
    # warm-up: every scene once through each server (pinned buffers of every
    # size, plan and queue buffers at their largest), then a short trace
    for srv in (plain, batched):
        for tk in [srv.submit(sc) for sc in scenes]:
            srv.wait(tk)
        serve_trace(srv, scenes, 200, 64, 99)

    def entry(k, rate, n):
        return {"rate_req_s": rate, "requests": n, "images_per_s": k["imagesPerS"], "p50_ms": k["p50Ms"],
                "p99_ms": k["p99Ms"], "p999_ms": k["p999Ms"], "mean_batch_images": k["meanBatchImages"],
                "failed": k["failed"], "peak_admitted_gb": k["peakAdmittedBytes"] / 1e9,
                "device_gb": k["deviceBytes"] / 1e9}

    for rate in rates:
        n = (400 if quick else 1000) if rate == 200 else 2000
        kp, res_p, _ = serve_trace(plain, scenes, rate, n, 7)
        kb, res_b, _ = serve_trace(batched, scenes, rate, n, 7)
        serving[f"rate_{rate}"] = {
            "plain": entry(kp, rate, n), "batched": entry(kb, rate, n),
            "identical": all(a.tobytes() == b.tobytes() for a, b in zip(res_p, res_b)),
            "images_per_s_ratio": kb["imagesPerS"] / kp["imagesPerS"],
            "p99_ratio": kb["p99Ms"] / kp["p99Ms"] if kp["p99Ms"] > 0 else None}
    plain.close()
    batched.close()
    # what batching can gain at most: the same kernel runs both servers, so a
    # batch only recovers the idle SMs of small images and the gaps between
    # launches; the 256-scene batch against the same scenes one by one
    b256 = out["batch_256"]
    serving["batched_over_plain_bound"] = {
        "ratio": b256["batch_over_plain"],
        "plain_mp_per_ms": b256["megapixels"] / (b256["s_per_batch"] * b256["batch_over_plain"] * 1e3),
        "batched_mp_per_ms": b256["megapixels"] / (b256["s_per_batch"] * 1e3),
        "note": "saturated serving throughput ratio cannot exceed the batched/plain ratio of the same scenes"}
    out["serving"] = serving
    # ---- CPU baseline: the oracle's restatement of detectMultiScaleCpu on all host threads
    O = _oracle()
    thr = os.cpu_count() or 1
    t = time.perf_counter()
    O.detect(pool, st, sg, scene1080, norm_mode=0, threads=thr)
    cdt = time.perf_counter() - t
    t = time.perf_counter()
    O.detect(pool, st, sg, scene1080, norm_mode=0, threads=1)
    cdt1 = time.perf_counter() - t
    out["cpu_baseline"] = {"value": 1.0 / cdt, "unit": "images/s", "cores": thr, "kind": "port",
                           "sample": "one 1920x1080 scene through the oracle's restatement of detectMultiScaleCpu "
                                     f"(raw detections, no grouping), {cdt:.2f} s",
                           "one_core": {"value": 1.0 / cdt1, "unit": "images/s", "cores": 1,
                                        "sample": f"the same scene on one thread, {cdt1:.2f} s"}}
    return out


def run_detect_case(args):
    """One detection case alone (profiling runs): `plain1080` (the 1920x1080
    scene) or `batchN` (the first N of the 256 scenes in one batch); W warm-up
    and K timed calls, then one JSON line with the work counters."""
    import torch

    import cs677s26_gb300 as V
    case = args.detect_case
    pool = V.feature_pool(V.FeatureMode.Basic)
    st, sg = V.synth_cascade(2)
    e = V.FaceVisionEngine((24, 24), 1, 3840, 2160, False, 200000)
    assert e.setCascadeModel(pool, st, sg) == 0
    if args.detect_config:
        assert e.setConfig(**json.loads(args.detect_config)) == 0
    if case == "plain1080":
        scene = V.synth_scene(1, 1920, 1080, 40, 24, 300)
        call = lambda: e.detectMultiScale(scene, 1920, 1080, 1920)  # noqa: E731
    elif case.startswith("batch"):
        # batchN: the first N of the 256 scenes from pageable memory; batchNp:
        # the same from page-locked memory (as the bench's batch line)
        pinned = case.endswith("p")
        k = int(case[5:-1] if pinned else case[5:])
        rng = np.random.default_rng(3)
        scenes = []
        for i in range(k):
            t = rng.random()
            scenes.append(V.synth_scene(1000 + i, int(round(320 * 12 ** t)), int(round(240 * 9 ** t)), 5, 24, 300))
        if pinned:
            keep = [torch.from_numpy(sc).pin_memory() for sc in scenes]
            scenes = [t_.numpy() for t_ in keep]
        call = lambda: e.detectBatch(scenes, capPerImage=4096)  # noqa: E731
    else:
        raise SystemExit(f"unknown detect case {case}")
    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        status, _ = call()
    dt = (time.perf_counter() - t) / max(1, args.steps)
    return {"detect_case": case, "config": e.getConfig(), "status": int(status), "ms_per_call": dt * 1e3,
            "stats": e.lastStats()}


# ----------------------------------------------------------------------------- CPU (oracle) arm
def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.lib()
    return O


def cpu_sample(O, pool, sums, inv, stride, threads):
    """One round of the oracle's restatement of runCpuWeakSearch over every
    `stride`-th feature of the pool (a sample spread over all positions,
    sizes and types); returns (seconds, features searched)."""
    feats = np.ascontiguousarray(pool[::stride])
    labels = np.array([1] * NPOS + [-1] * NNEG, np.int8)
    w = np.where(labels > 0, np.float32(0.5) / np.float32(NPOS), np.float32(0.5) / np.float32(NNEG)).astype(np.float32)
    t = time.perf_counter()
    O.weak_search(feats, sums, inv, labels, w, threads=threads)
    return time.perf_counter() - t, len(feats)


def cpu_baseline(target_s=15.0):
    """The oracle's restatement of runCpuWeakSearch on all host threads (and on
    one), over a feature sample spread across the pool, scaled by the 20 B
    model to the metric's unit."""
    O = _oracle()
    pool = O.feature_pool(0)
    sums, inv = O.train_integrals(O.synth_patches(SEED, NPOS, NNEG))
    n = NPOS + NNEG
    threads = os.cpu_count() or 1
    stride = max(1, len(pool) // (64 * threads))
    dt, nf = cpu_sample(O, pool, sums, inv, stride, threads)
    stride = max(1, int(stride * dt / target_s))
    dt, nf = cpu_sample(O, pool, sums, inv, stride, threads)
    gbs = BYTES_PER_ELEM_ROUND * nf * n / dt / 1e9
    # the reference's CPU search is single-threaded: the same search on one core
    stride1 = max(1, int(stride * threads * dt / 3.0))
    dt1, nf1 = cpu_sample(O, pool, sums, inv, stride1, 1)
    return {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"one round of the oracle's restatement of runCpuWeakSearch over every {stride}-th of the "
                      f"162,336 features ({nf} features) x {n} samples ({dt:.1f} s, {threads} threads), scaled by "
                      "the 20 B model",
            "one_core": {"value": BYTES_PER_ELEM_ROUND * nf1 * n / dt1 / 1e9, "unit": "GB/s", "cores": 1,
                         "sample": f"every {stride1}-th feature ({nf1}) x {n} samples ({dt1:.1f} s, 1 thread)"}}


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores, through the oracle (its
    restatement of runCpuWeakSearch and detectMultiScaleCpu; the reference's
    own sources are not on the GPU machines).  Inputs come from the oracle's
    generators, byte-identical to the package's; nothing of the package is
    loaded.  Each step is one round over a feature sample spread across the
    whole pool (every k-th feature), sized to a few seconds."""
    if rank != 0:
        return None
    O = _oracle()
    pool = O.feature_pool(0)
    patches = O.synth_patches(SEED, NPOS, NNEG)
    sums, inv = O.train_integrals(patches)
    threads = os.cpu_count() or 1
    n = len(patches)
    stride = max(1, len(pool) // (128 * threads))
    for _ in range(args.warmup):
        cpu_sample(O, pool, sums, inv, stride * 4, threads)
    runs = [cpu_sample(O, pool, sums, inv, stride, threads) for _ in range(args.steps)]
    dt = sum(r[0] for r in runs) / len(runs)
    nfeat = runs[0][1]
    value = BYTES_PER_ELEM_ROUND * nfeat * n / dt / 1e9
    # detection: the oracle's restatement of detectMultiScaleCpu on the 1920x1080 scene
    st, sg = O.synth_cascade(2)
    scene = O.synth_scene(1, 1920, 1080, 40, 24, 300)
    t = time.perf_counter()
    raw = O.detect(pool, st, sg, scene, norm_mode=0, threads=threads)
    cdt = time.perf_counter() - t
    return {
        "detect": {"plain_1080p": {"images_per_s": 1.0 / cdt, "ms_per_image": cdt * 1e3, "cores": threads,
                                   "raw_detections": int(len(raw))}},
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": DTYPE, "data": "synthetic",
        "config": workload_config(len(pool), n, world),
        "sample": {"features_per_step": nfeat, "feature_stride": stride, "rounds_per_step": 1,
                   "scaled_to": "the 20 B per feature-sample per round model of the same workload"},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"every {stride}-th of the 162,336 features ({nfeat}) x {n} samples per step "
                                   "(the oracle's restatement of runCpuWeakSearch; the reference's sources are not "
                                   "on this machine)"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--features", type=int, default=162336, help="first K Basic features (profiling cases)")
    ap.add_argument("--rounds", type=int, default=50, help="boosting rounds per step (profiling cases)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-detect", action="store_true", help="stump step only")
    ap.add_argument("--quick-detect", action="store_true", help="shorter serving traces")
    ap.add_argument("--detect-case", default=None,
                    help="run one detection case alone: plain1080, batchN (pageable scenes) or batchNp (page-locked)")
    ap.add_argument("--detect-config", default=None, help="launch shape for --detect-case, as JSON")
    args = ap.parse_args()
    global ROUNDS
    ROUNDS = args.rounds
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.detect_case:
        res = run_detect_case(args)
    elif args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_gpu(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
