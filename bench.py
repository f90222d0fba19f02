#!/usr/bin/env python3
"""Benchmark of the CMP/CRS semblance search on one GB300 (or N, one rank per GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

A step is one whole search of the workload (every CDP x t0 x candidate) through
semb_plan_run, inputs resident in HBM.  The default workload is the 4,096-CMP
uneven-fold CMP line (fold 12-240, ns 2000 at 2 ms, 256 velocities, tau 4 ms)
searched with the batched form and FP16 trace storage; the plain FP32 form runs on
the same data for comparison.  Prints one JSON line.

value        batched evals/s (CDP x t0 x candidate), whole job over N GPUs
e2e          the same metric through the public C ABI from pinned host buffers:
             semb_plan_stream (H2D copies of CDP chunks overlapped with the search,
             device binning) + semb_plan_download (D2H of ctr/str/stk) every step;
             upload_then_run: semb_plan_upload + semb_plan_run + download instead
roofline     the search kernel against the FP32 FMA rate measured live by
             semb_probe_fp32 (the kernels are bound by FP32 issue, not HBM)
cpu_baseline the oracle (CPU restatement of the reference's OpenMP search) on a
             bounded sample of the workload, all host threads
target       (N = 1) the batched-vs-plain goal on the 20,000-CDP uneven-aperture CRS
             survey (FP16 store, 21^3 grid): one timed step of each form with CUDA
             events, the ratio, and the batched form's error against the FP64
             oracle on a seeded sample of CDPs from every aperture bucket

With N > 1 (torchrun, one rank per GPU) rank r searches segment r of the survey
(synth.config(..., segment=r): the same shapes from another seed, placed apart):
per-GPU work is fixed as N grows (weak scaling) and no data crosses ranks.

--impl reference times the reference's own CPU implementation of the path instead:
the reference's OpenMP programs in oracle/_ref where they were built on this
machine, else the oracle restatement, which reproduces them bit for bit.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ipdps-crs-cmp-code_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

import semb  # noqa: E402
import synth  # noqa: E402

METRIC = "CRS/CMP semblance evals/s on 1 GB300: batched FP16-store vs plain FP32, at error"

WORKLOADS = {
    # name: (generator config index, default CDP count, method)
    "cmp-4096-uneven": (1, None, semb.CMP),
    "cmp-200x60": (0, None, semb.CMP),
    "crs-500x48": (2, None, semb.CRS),
    "crs-uneven-2000": (3, 2000, semb.CRS),
    "crs-uneven-20k": (3, None, semb.CRS),
    # the 100k-CDP, 31^3-grid survey with BF16 traces; --ncdp runs its first N CDPs
    "crs-100k-31cubed": (4, 1000, semb.CRS),
}
# trace storage of the workloads whose survey names one (else --storage, f16)
WORKLOAD_STORAGE = {"crs-100k-31cubed": "bf16"}

SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- data

TARGET_WORKLOAD = "crs-uneven-20k"
TARGET_RATIO = 3.0


def make_gather(name: str, ncdp: int | None, segment: int = 0):
    """Synthetic survey of a workload; traces are CDP-major, so cdp_end follows
    from the folds.  Rank r of a multi-GPU run gets segment r (weak scaling)."""
    idx, n_default, method = WORKLOADS[name]
    s = synth.config(idx, ncdp=ncdp or n_default, segment=segment)
    cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
    return s, method, cdp_end, s.headers


def window_of(s) -> int:
    """w = 2*tau+1 with the reference's single-precision rule
    (CRS/OpenMP/src/main.cpp:135-138)."""
    dt = np.float32(np.float32(int(s.headers["dt"][0])) / np.float32(1000000.0))
    idt = np.float32(np.float32(1.0) / dt)
    tau = int(np.float32(np.float32(float(s.params["tau"])) * idt))
    return 2 * max(tau, 0) + 1


L2_BYTES = 129e6   # GB300 L2 cache


def workload_config(name: str, s, method: int, world: int, mean_aperture: float | None) -> dict:
    """The `config` of both arms' JSON lines: the workload and its sizes."""
    ncand = int(s.params["nc"]) if method == semb.CMP else int(s.params["na"] * s.params["nb"] * s.params["nc"])
    ncdp = int(s.info["ncdp"])
    cfg = {"workload": name, "name": s.name, "ncdps": ncdp * world, "ns": s.ns, "ncand": ncand,
           "window": window_of(s), "traces": s.ntraces * world,
           "parallelism": (f"survey segments x{world} (one per rank, no collective)" if world > 1
                           else "single GPU"),
           "l2": ("inputs larger than L2 (FP32 %.2f GB, FP16 %.2f GB per GPU)" if s.samples.nbytes / 2 > L2_BYTES
                  else "inputs within L2, no flush between steps (FP32 %.2f GB, FP16 %.2f GB per GPU)")
                 % (s.samples.nbytes / 1e9, s.samples.nbytes / 2e9)}
    if mean_aperture is not None:
        cfg["mean_aperture"] = mean_aperture
        cfg["trace_evals_per_step"] = int(round(mean_aperture * ncdp * world)) * s.ns * ncand
    return cfg


def mean_aperture_host(s, method) -> float:
    """Aperture traces per CDP averaged over the survey (CMP: the fold; CRS: the
    folds of every CDP within apm of the first-trace midpoint)."""
    folds = np.asarray(s.info["fold"], np.int64)
    if method == semb.CMP:
        return float(folds.mean())
    import shard
    cdp_end = np.cumsum(folds)
    first = np.concatenate([[0], cdp_end[:-1]])
    mx, my = shard.first_trace_midpoints({k: s.headers[k][first] for k in ("gx", "gy", "sx", "sy", "scalco")})
    ap = [folds[nb].sum() for nb in shard.neighbours_of(mx, my, s.params["apm"], range(len(folds)))]
    return float(np.mean(ap))


def gather_arrays(s, cdp_end, samples=None):
    h = s.headers
    return semb.GatherArrays(cdp_end, s.ns, int(h["dt"][0]), h["gx"], h["gy"], h["sx"], h["sy"], h["scalco"],
                             s.samples if samples is None else samples, cdp=np.arange(1, len(cdp_end) + 1))


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    def __init__(self, device: int):
        self.device, self.proc, self.out = device, None, None

    def __enter__(self):
        try:
            self.out = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + SMI_FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.proc or not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.out.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.out.read())) if len(r) >= 9]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for k, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- helpers

def algo_flops(method: int, st: dict, nap: int, lin: bool = True) -> float:
    """Algorithmic FLOPs of one search: per eval N_ap*(T + 7w) + 2w + 2 with T = 5
    (CMP: add, mul, sqrt, scale, frac) or 10 (CRS), per window sample 3 for the
    interpolation, 1 for num, 2 for den and 1 for the reference's linear sum (the
    algorithm's count, which `roofline.achieved` uses).  lin=False leaves the linear
    sum out: the batched form takes its stack from the numerators, so this is the
    count of the operations it performs (`roofline.achieved_own_ops`).  Both count the
    traces that no item of a pass can reach, which the kernel skips (about 1-2% of the
    trace-evaluations on the CRS surveys)."""
    w = st["window"]
    T = 5 if method == semb.CMP else 10
    per_cand_t0 = nap * (T + (7 if lin else 6) * w) + st["ncdps"] * (2 * w + 2)
    return float(st["ns"]) * st["ncand"] * per_cand_t0


def fp32_roofline(method: int, st: dict, nap: int, ms: float, peak: float) -> dict:
    """The FP32 side of the roofline of a batched search that took `ms`: the
    algorithm's FLOP/s and the batched form's own, against the live FMA-rate probe."""
    ach = algo_flops(method, st, nap) / (ms * 1e-3) / 1e12
    own = algo_flops(method, st, nap, lin=False) / (ms * 1e-3) / 1e12
    return {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "achieved_own_ops": own, "frac_own_ops": own / peak,
            "peak_source": "measured live: semb_probe_fp32 FMA throughput"}


def timed_runs(plan: semb.Plan, warmup: int, steps: int):
    for _ in range(warmup):
        plan.run()
    dev_ms, t0 = [], time.perf_counter()
    search_ms = []
    for _ in range(steps):
        plan.run()
        st = plan.stats()
        dev_ms.append(st["ms_total"])
        search_ms.append(st["ms_search"])
    wall = time.perf_counter() - t0
    return dev_ms, search_ms, wall, plan.stats()


def traffic_from_profiles(workload: str, ncdps: int, trace_evals: int):
    """DRAM bytes per search launch from the single-pass ncu captures summarised in
    profiles/traffic.json: the captured figure when the workload and CDP count match,
    else that capture scaled by trace-evaluations (the staged windows and the top-4
    outputs grow with the CDPs searched).  None when no capture covers the workload."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            table = json.load(f)
    except (OSError, ValueError):
        return None
    e = table.get(workload)
    if e is None:
        return None
    src = table.get(e["scaled_from"]) if "scaled_from" in e else e
    if not src or "dram_read" not in src:
        return None
    captured = src["dram_read"] + src["dram_write"]
    if "scaled_from" not in e and src["ncdps"] == ncdps:
        return float(captured)
    return float(captured) * trace_evals / src["trace_evals"]


def smem_from_profiles(workload: str):
    """Shared-memory load wavefronts of the search kernel, % of peak, from the ncu
    capture summarised in profiles/ (None when no capture covers the workload)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            table = json.load(f)
    except (OSError, ValueError):
        return None
    e = table.get(workload) or {}
    src = table.get(e.get("scaled_from", ""), e)
    if "smem_load_wavefronts_pct_of_peak" not in src:
        return None
    return {"load_wavefronts_pct_of_peak": src["smem_load_wavefronts_pct_of_peak"], "source": src["smem_source"]}


def oracle_mod():
    if ORACLE_DIR not in sys.path:
        sys.path.insert(0, ORACLE_DIR)
    import oracle  # noqa: E402  (checker / CPU baseline only)
    return oracle


def sub_gather(oracle, s, method, cdp_end, idx, precision):
    """The oracle's gather of the CDPs in idx plus, for CRS, every CDP within apm of
    one of them (their halo): the sampled CDPs then have their whole apertures, in
    the reference's order, and the search costs only the sample.  Returns the gather
    and the sampled CDPs' positions in it."""
    real = np.float32 if precision == "f32" else np.float64
    idx = np.asarray(idx, np.int64)
    if method == semb.CRS:
        import shard
        first = np.concatenate([[0], cdp_end[:-1]])
        mx, my = shard.first_trace_midpoints({k: s.headers[k][first] for k in ("gx", "gy", "sx", "sy", "scalco")})
        need = np.unique(np.concatenate(shard.neighbours_of(mx, my, s.params["apm"], idx) + [idx]))
    else:
        need = np.unique(idx)
    starts = np.concatenate([[0], cdp_end[:-1]])
    rows = np.concatenate([np.arange(starts[i], cdp_end[i]) for i in need])
    g = oracle.gather(s.headers[rows], s.samples[rows], "cmp" if method == semb.CMP else "crs", s.params["aph"],
                      s.params.get("apm"), real=real)
    return g, np.searchsorted(need, idx)


def oracle_search(oracle, g, s, method, precision, cdps, t0_range=None, top2=False, threads=0):
    fn = oracle.cmp if method == semb.CMP else oracle.crs
    return fn(g, s.params, precision, threads=threads, cdps=cdps, t0_range=t0_range, top2=top2)


def bucket_sample(aperture: np.ndarray, per_bucket: int, seed: int, big: int = 1500, nbig: int = 2) -> np.ndarray:
    """Seeded CDP sample with `per_bucket` CDPs from each aperture bucket of the
    plan's work queue (> 1024, 385-1024, 129-384, <= 128 aperture traces), at
    least `nbig` of them with `big` or more aperture traces where the survey has
    such CDPs."""
    rng = np.random.default_rng(seed)
    edges = [(1025, 1 << 30), (385, 1024), (129, 384), (0, 128)]
    out = []
    for lo, hi in edges:
        cand = np.nonzero((aperture >= lo) & (aperture <= hi))[0]
        if len(cand) == 0:
            continue
        pick = list(rng.choice(cand, size=min(per_bucket, len(cand)), replace=False))
        if lo == 1025:
            bigs = np.nonzero(aperture >= big)[0]
            have = sum(int(aperture[i] >= big) for i in pick)
            if len(bigs) and have < nbig:
                extra = [int(i) for i in rng.choice(bigs, size=min(nbig, len(bigs)), replace=False) if i not in pick]
                pick = extra[:nbig - have] + pick[:max(0, len(pick) - (nbig - have))]
        out += [int(i) for i in pick]
    return np.array(sorted(set(out)), np.int64)


def cpu_rate(oracle, s, method, cdp_end, n_sample, seed, threads=0):
    """The oracle (single precision, the reference's arithmetic) on a seeded sample
    of CDPs, timed by its own clock, which like the reference's excludes I/O;
    returns (evals/s, seconds, sample text)."""
    ncdp = len(cdp_end)
    rng = np.random.default_rng(seed)
    if method == semb.CMP:
        idx = np.sort(rng.choice(ncdp, size=min(n_sample, ncdp), replace=False))
        text = f"{len(idx)} seeded-random CMPs of {ncdp}"
    else:
        start = int(rng.integers(0, max(1, ncdp - n_sample)))
        idx = np.arange(start, min(ncdp, start + n_sample))
        text = f"{len(idx)} contiguous CDPs of {ncdp}"
    g, local = sub_gather(oracle, s, method, cdp_end, idx, "f32")
    out = oracle_search(oracle, g, s, method, "f32", local, threads=threads)
    ncand = int(s.params["nc"]) if method == semb.CMP else int(s.params["na"] * s.params["nb"] * s.params["nc"])
    evals = len(idx) * s.ns * ncand
    return evals / out["seconds"], out["seconds"], text


def errors_vs_fp64(oracle, s, method, cdp_end, outs: dict, idx, t0_blocks=None, seed=7):
    """Errors of each form's results (outs: name -> (ctr, sem, stk) over the whole
    survey) against the FP64 oracle on the CDPs in idx, over every t0 or over
    `t0_blocks` seeded blocks of 32 t0 per CDP: max |semblance| and |stack| error,
    identical picks over all sampled (CDP, t0) and over those whose FP64 best two
    semblances differ by more than 1e-6."""
    g, local = sub_gather(oracle, s, method, cdp_end, idx, "f64")
    ns = s.ns
    if t0_blocks is None:
        ranges = [(0, ns)]
    else:
        rng = np.random.default_rng(seed)
        nblk = (ns + 31) // 32
        ranges = [(32 * int(b), min(ns, 32 * int(b) + 32))
                  for b in np.sort(rng.choice(nblk, size=min(t0_blocks, nblk), replace=False))]
    rows_t0 = []
    ref = {"ctr": [], "str": [], "stk": [], "top2": []}
    secs = 0.0
    for lo, hi in ranges:
        o = oracle_search(oracle, g, s, method, "f64", local, t0_range=(lo, hi), top2=True)
        secs += o["seconds"]
        for k in ref:
            ref[k].append(o[k][local, lo:hi])
        rows_t0.append(np.arange(lo, hi))
    ref = {k: np.concatenate(v, axis=1) for k, v in ref.items()}
    t0s = np.concatenate(rows_t0)
    decisive = ref["top2"] > 1e-6
    res = {"sample": (f"{len(idx)} CDPs ({'every t0' if t0_blocks is None else f'{len(t0s)} t0 in {len(ranges)} '
                                            f'seeded blocks'}), FP64 oracle"),
           "pairs": int(ref["ctr"].size), "decisive_pairs": int(decisive.sum()), "oracle_s": secs}
    for name, (ctr, sem, stk) in outs.items():
        c, sm, sk = (a[np.ix_(idx, t0s)] for a in (ctr, sem, stk))
        same = c == ref["ctr"]
        res[name] = {"sem_max_abs": float(np.max(np.abs(sm - ref["str"]))),
                     "stack_max_abs": float(np.max(np.abs(sk - ref["stk"]))),
                     # a differing pick stacks along another candidate's traveltime
                     "stack_max_abs_same_pick": float(np.max(np.abs(sk - ref["stk"])[same])) if same.any() else None,
                     "identical_picks": float(same.mean()),
                     "identical_picks_decisive": float(same[decisive].mean()) if decisive.any() else None}
    return res


# ----------------------------------------------------------------------------- arms

def run_reference_arm(args, rank, world):
    """The reference's CPU implementation of the path on the host cores, rank 0
    only: the reference's own OpenMP program where oracle/_ref was built on this
    machine (timed by its INFO line), else the oracle restatement (timed by its
    own clock, which excludes I/O like the reference's)."""
    if rank != 0:
        return 0
    s, method, cdp_end, _ = make_gather(args.workload, args.ncdp)
    oracle = oracle_mod()
    threads = os.cpu_count() or 1
    n_sample = args.cpu_sample or (96 if method == semb.CMP else 8)
    ncand = int(s.params["nc"]) if method == semb.CMP else int(s.params["na"] * s.params["nb"] * s.params["nc"])
    use_ref = oracle.have_reference()
    kind = "reference" if use_ref else "port"
    vals = []
    text = ""
    for step in range(args.warmup + args.steps):
        if use_ref:
            rate, text = ref_program_rate(oracle, s, method, cdp_end, n_sample, seed=step, threads=threads)
        else:
            rate, _, text = cpu_rate(oracle, s, method, cdp_end, n_sample, seed=step, threads=threads)
        if step >= args.warmup:
            vals.append(rate)
    value = statistics.median(vals)
    ms = s.ns * n_sample * ncand / value * 1e3
    what = ("the reference's own OpenMP program (oracle/_ref), rate from its INFO line" if use_ref
            else "CPU restatement of the reference's OpenMP search, bit-identical to it")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.workload, s, method, 1, mean_aperture_host(s, method)),
            "sample_per_step": text,
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": kind,
                             "sample": f"{text} per step ({what})"},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def ref_program_rate(oracle, s, method, cdp_end, n_sample, seed, threads):
    """Run the reference's own program (oracle/_ref) on an SU file of a seeded CDP
    sample (CRS: with the sample's halo, searching every CDP of the file) and take
    its rate from its INFO line's execution time."""
    import su
    rng = np.random.default_rng(seed)
    ncdp = len(cdp_end)
    if method == semb.CMP:
        idx = np.sort(rng.choice(ncdp, size=min(n_sample, ncdp), replace=False))
    else:
        start = int(rng.integers(0, max(1, ncdp - n_sample)))
        idx = np.arange(start, min(ncdp, start + n_sample))
    starts = np.concatenate([[0], cdp_end[:-1]])
    rows = np.concatenate([np.arange(starts[i], cdp_end[i]) for i in idx])
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.su")
        su.write_su(path, s.headers[rows], s.samples[rows])
        args = s.cli_args(path)[:-2]
        out = oracle.run_reference("cmp" if method == semb.CMP else "crs", "f32", path, args, threads=threads,
                                   workdir=d)
    import re
    m = re.search(r"Execution Time:\s*([0-9.eE+-]+)", out["info"])
    if not m:
        raise RuntimeError(f"no execution time in the reference's output: {out['info']!r}")
    secs = float(m.group(1))
    ncand = int(s.params["nc"]) if method == semb.CMP else int(s.params["na"] * s.params["nb"] * s.params["nc"])
    return len(idx) * s.ns * ncand / secs, f"{len(idx)} CDPs of {ncdp} in one SU file"


def run_target(args, dev):
    """The goal on the 20,000-CDP CRS survey: one timed batched step (FP16 store,
    search + FP64 re-pick) against one timed plain FP32 step on the same GPU, and
    the batched form's error against the FP64 oracle."""
    t_gen = time.perf_counter()
    s, method, cdp_end, _ = make_gather(TARGET_WORKLOAD, args.target_ncdp)
    log(f"[target] generated {s.ntraces} traces x {s.ns} samples in {time.perf_counter() - t_gen:.1f}s")
    arrays = gather_arrays(s, cdp_end)
    out = {"workload": TARGET_WORKLOAD, "name": s.name, "storage": "f16", "ncdps": int(len(cdp_end)),
           "traces": s.ntraces, "goal_ratio": TARGET_RATIO}
    with semb.Plan(semb.params(method, mode=semb.BATCHED, storage=semb.STORE_F16, **s.params), device=dev) as bp:
        bp.upload(arrays.view())
        bp.use_graph(False)
        bp.run()
        st = bp.stats()
        ap = bp.download_attrs(batched=False)["aperture"]
        b_out = bp.download()
    nap = int(ap.sum())
    out.update(ncand=st["ncand"], window=st["window"], mean_aperture=float(ap.mean()),
               evals=st["evals"], trace_evals=st["trace_evals"], variant=st["variant"])
    out["batched"] = {"ms": st["ms_total"], "ms_search": st["ms_search"], "ms_repick": st["ms_repick"],
                      "repicked": st["repicked"], "evals_per_s": st["evals"] / (st["ms_total"] * 1e-3)}
    log(f"[target] batched {st['ms_total']:.0f} ms")
    with semb.Plan(semb.params(method, mode=semb.PLAIN_F32, **s.params), device=dev) as pp:
        pp.upload(arrays.view())
        pp.run()
        pst = pp.stats()
        p_out = pp.download()
    log(f"[target] plain {pst['ms_total']:.0f} ms")
    out["plain"] = {"ms": pst["ms_total"], "evals_per_s": pst["evals"] / (pst["ms_total"] * 1e-3)}
    out["ratio"] = pst["ms_total"] / st["ms_total"]
    out["met"] = bool(out["ratio"] >= TARGET_RATIO)
    out["roofline"] = fp32_roofline(method, st, nap, st["ms_search"], semb.probe_fp32_tflops(dev))
    if not args.no_cpu:
        oracle = oracle_mod()
        idx = bucket_sample(ap, per_bucket=args.target_err_per_bucket, seed=11)
        t_err = time.perf_counter()
        out["error_vs_fp64"] = errors_vs_fp64(oracle, s, method, cdp_end, {"batched": b_out, "plain": p_out}, idx,
                                              t0_blocks=args.target_t0_blocks, seed=13)
        out["error_vs_fp64"]["apertures"] = sorted(int(ap[i]) for i in idx)
        log(f"[target] FP64 errors on {len(idx)} CDPs in {time.perf_counter() - t_err:.0f}s")
    return out


def run_chunked_survey(args):
    """A whole survey in CDP chunks, each chunk's search + re-pick one CUDA graph
    (semb_plan_set_chunks), one run; with the batched form's error against the FP64
    oracle on a seeded sample of CDPs.  The oracle runs in a child process forked
    before the first GPU call, on the host cores, while the GPU searches."""
    t_gen = time.perf_counter()
    s, method, cdp_end, _ = make_gather(args.workload, args.ncdp)
    ncdp = len(cdp_end)
    log(f"[chunked] generated {ncdp} CDPs, {s.ntraces} traces x {s.ns} samples in {time.perf_counter() - t_gen:.0f}s")
    storage = {"f16": semb.STORE_F16, "bf16": semb.STORE_BF16, "f32": semb.STORE_F32}[args.storage]
    rng = np.random.default_rng(args.err_seed)
    n_err = max(1, int(round(ncdp * args.err_frac)))
    idx = np.sort(rng.choice(ncdp, size=min(n_err, ncdp), replace=False))
    nblk = (s.ns + 31) // 32
    blocks = np.sort(rng.choice(nblk, size=min(args.err_t0_blocks, nblk), replace=False))
    child, err_path = None, None
    if not args.no_cpu:
        err_path = tempfile.mktemp(prefix="semb_c4_oracle_", suffix=".npz")
        child = os.fork()
        if child == 0:   # CPU only: the FP64 oracle on the sample, then exit
            try:
                oracle = oracle_mod()
                g, local = sub_gather(oracle, s, method, cdp_end, idx, "f64")
                parts = {k: [] for k in ("ctr", "str", "stk", "top2")}
                secs = 0.0
                for b in blocks:
                    lo, hi = 32 * int(b), min(s.ns, 32 * int(b) + 32)
                    o = oracle_search(oracle, g, s, method, "f64", local, t0_range=(lo, hi), top2=True)
                    secs += o["seconds"]
                    for k in parts:
                        parts[k].append(o[k][local, lo:hi])
                np.savez(err_path, secs=secs, **{k: np.concatenate(v, axis=1) for k, v in parts.items()})
                os._exit(0)
            except BaseException as e:   # noqa: BLE001
                print(f"[chunked] oracle child failed: {e!r}", file=sys.stderr, flush=True)
                os._exit(1)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    out = {"workload": args.workload, "name": s.name, "storage": args.storage, "ncdps": ncdp, "traces": s.ntraces,
           "chunk_cdps": args.chunk_cdps}
    with semb.Plan(semb.params(method, mode=semb.BATCHED, storage=storage, **s.params), device=dev) as plan:
        t_up = time.perf_counter()
        plan.upload(gather_arrays(s, cdp_end).view())
        out["upload_s"] = time.perf_counter() - t_up
        if args.variant is not None:
            plan.set_variant(args.variant)
            out["variant"] = args.variant
        elif args.tune:
            t_tune = time.perf_counter()
            v, ms = plan.autotune()
            out["autotune"] = {"variant": v, "sample_ms": ms, "seconds": time.perf_counter() - t_tune,
                               "buckets": [dict(zip(("ap_lo", "ap_hi", "tasks", "variant"), b))
                                           for b in plan.buckets()]}
        plan.set_chunks(args.chunk_cdps)
        with ClockSampler(dev) as clk:
            plan.run()
        st = plan.stats()
        chunk_ms = plan.chunk_times()
        ap = plan.download_attrs(batched=False)["aperture"]
        ctr, sem, stk = plan.download()
    nap = int(ap.sum())
    total_ms = st["ms_total"]
    roof = fp32_roofline(method, st, nap, total_ms, semb.probe_fp32_tflops(dev))
    roof["note"] = "search + re-pick time of every chunk (graph replays give no split)"
    out.update(ncand=st["ncand"], window=st["window"], mean_aperture=float(ap.mean()), evals=st["evals"],
               trace_evals=st["trace_evals"], ms_total=total_ms, chunks=len(chunk_ms), ms_per_chunk=chunk_ms,
               evals_per_s=st["evals"] / (total_ms * 1e-3), repicked=st["repicked"],
               kernel_launches=st["kernel_launches"], clocks=clk.summary(),
               roofline=roof)
    if child is not None:
        _, status = os.waitpid(child, 0)
        if status == 0 and os.path.exists(err_path):
            ref = np.load(err_path)
            t0s = np.concatenate([np.arange(32 * int(b), min(s.ns, 32 * int(b) + 32)) for b in blocks])
            c, sm, sk = (a[np.ix_(idx, t0s)] for a in (ctr, sem, stk))
            same = c == ref["ctr"]
            decisive = ref["top2"] > 1e-6
            out["error_vs_fp64"] = {
                "sample": f"{len(idx)} seeded CDPs ({args.err_frac:.1%}) x {len(t0s)} t0 in {len(blocks)} blocks, "
                          f"FP64 oracle ({float(ref['secs']):.0f} s on the host cores)",
                "pairs": int(same.size), "decisive_pairs": int(decisive.sum()),
                "sem_max_abs": float(np.max(np.abs(sm - ref["str"]))),
                "stack_max_abs": float(np.max(np.abs(sk - ref["stk"]))),
                "stack_max_abs_same_pick": float(np.max(np.abs(sk - ref["stk"])[same])) if same.any() else None,
                "identical_picks": float(same.mean()),
                "identical_picks_decisive": float(same[decisive].mean()) if decisive.any() else None}
            os.unlink(err_path)
        else:
            out["error_vs_fp64"] = {"failed": f"oracle child exit status {status}"}
    print(json.dumps({"chunked_survey": out}), flush=True)
    return 0


def run_ours(args, rank, world, dist):
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    t_gen = time.perf_counter()
    s, method, cdp_end, _ = make_gather(args.workload, args.ncdp, segment=rank if world > 1 else 0)
    log(f"[rank {rank}] generated {s.ntraces} traces x {s.ns} samples in {time.perf_counter() - t_gen:.1f}s")
    # pinned host copy of the samples for the end-to-end leg
    pinned = semb.PinnedArray(s.samples.shape, np.float32)
    pinned.array[...] = s.samples
    arrays = gather_arrays(s, cdp_end, pinned.array)
    nap = None
    res = {}

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    storage = {"f16": semb.STORE_F16, "bf16": semb.STORE_BF16, "f32": semb.STORE_F32}[args.storage]
    gap = {} if args.repick_gap is None else {"repick_gap": args.repick_gap}
    plan = semb.Plan(semb.params(method, mode=semb.BATCHED, storage=storage, **gap, **s.params), device=dev)
    plan.upload(arrays.view())
    if args.variant is not None:
        plan.set_variant(args.variant)
    tune = plan.autotune() if args.tune and args.variant is None else None
    buckets = plan.buckets()
    st0 = plan.stats()
    nap = int(round(st0["trace_evals"] / (st0["ns"] * st0["ncand"])))
    # per-kernel split (search vs re-pick) from direct launches
    plan.use_graph(False)
    _, search_ms, _, st_direct = timed_runs(plan, 1, 2)
    plan.use_graph(bool(args.graph))
    barrier()
    with ClockSampler(dev) as clk:
        dev_ms, _, wall, st = timed_runs(plan, args.warmup, args.steps)
    barrier()
    total_ms = max_over_ranks(sum(dev_ms))
    evals = st["evals"]
    value = world * evals * args.steps / (total_ms * 1e-3)
    ms_search = statistics.mean(search_ms)
    flops = algo_flops(method, st, nap)
    res["batched"] = dict(ms=sum(dev_ms) / args.steps, ms_search=ms_search, ms_repick=st_direct["ms_repick"],
                          repicked=st["repicked"], wall_s=wall, launches=st["kernel_launches"])

    # the same search in the plain FP32 form
    plain = semb.Plan(semb.params(method, mode=semb.PLAIN_F32, **s.params), device=dev)
    plain.upload(arrays.view())
    p_ms, p_search, p_wall, pst = timed_runs(plain, 1, max(1, args.steps))
    plain_ms = max_over_ranks(sum(p_ms)) / max(1, args.steps)
    res["plain"] = dict(ms=plain_ms, value=world * evals / (plain_ms * 1e-3))

    # other storage forms, briefly
    for name, stv in (("bf16", semb.STORE_BF16), ("f32", semb.STORE_F32)):
        if args.quick or name == args.storage:
            continue
        with semb.Plan(semb.params(method, mode=semb.BATCHED, storage=stv, **s.params), device=dev) as p2:
            p2.upload(arrays.view())
            a_ms, *_ = timed_runs(p2, 1, 2)
            res["store_" + name] = dict(ms=sum(a_ms) / 2, value=evals / (sum(a_ms) / 2 * 1e-3))

    # end to end through the public API: upload from pinned memory + run + download
    e2e = None
    if not args.no_e2e:
        ctr = semb.PinnedArray((st["ncdps"] * st["ns"],), np.int32)
        sem = semb.PinnedArray((st["ncdps"] * st["ns"],), np.float32)
        stk = semb.PinnedArray((st["ncdps"] * st["ns"],), np.float32)
        plan.use_graph(False)
        for _ in range(1):
            plan.upload(arrays.view())
            plan.run()
            plan.download(ctr.array, sem.array, stk.array)
        barrier()
        t0 = time.perf_counter()
        phase = [0.0, 0.0, 0.0]   # upload, run, download (host wall time)
        up_dev = 0.0              # upload's device time (CUDA events)
        for _ in range(args.steps):
            ta = time.perf_counter()
            plan.upload(arrays.view())
            tb = time.perf_counter()
            plan.run()
            tc = time.perf_counter()
            plan.download(ctr.array, sem.array, stk.array)
            td = time.perf_counter()
            phase[0] += tb - ta
            phase[1] += tc - tb
            phase[2] += td - tc
            up_dev += plan.stats()["ms_upload"]
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        h2d = s.samples.nbytes + 5 * 4 * s.ntraces + 8 * len(cdp_end)
        d2h = 3 * 4 * st["ncdps"] * st["ns"]
        # streamed: semb_plan_stream overlaps the trace copies with the search
        plan.stream(arrays.view(), args.stream_chunks)
        plan.download(ctr.array, sem.array, stk.array)
        barrier()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            plan.stream(arrays.view(), args.stream_chunks)
            plan.download(ctr.array, sem.array, stk.array)
        s_s = max_over_ranks(time.perf_counter() - t1)
        e2e = {"value": world * evals * args.steps / s_s, "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": s_s / args.steps * 1e3,
               "api": f"semb_plan_stream ({args.stream_chunks} chunks) + semb_plan_download",
               "upload_then_run": {"value": world * evals * args.steps / e2e_s, "ms_per_step": e2e_s / args.steps * 1e3,
                                   "ms_upload": phase[0] / args.steps * 1e3,
                                   "ms_upload_device": up_dev / args.steps,
                                   "ms_run": phase[1] / args.steps * 1e3,
                                   "ms_download": phase[2] / args.steps * 1e3}}
        ctr.free(), sem.free(), stk.free()

    # error of both forms against the FP64 oracle on a sample, and the CPU baseline
    err = None
    cpu = None
    if rank == 0 and not args.no_cpu:
        oracle = oracle_mod()
        b_out = plan.download()
        p_out = plain.download()
        ap = plan.download_attrs(batched=False)["aperture"]
        if method == semb.CMP:
            idx = bucket_sample(ap, per_bucket=8, seed=7)
            err = errors_vs_fp64(oracle, s, method, cdp_end, {"batched": b_out, "plain": p_out}, idx)
        else:
            idx = bucket_sample(ap, per_bucket=4, seed=7)
            err = errors_vs_fp64(oracle, s, method, cdp_end, {"batched": b_out, "plain": p_out}, idx, t0_blocks=4)
        err["apertures"] = sorted(int(ap[i]) for i in idx)
        threads = os.cpu_count() or 1
        n_cpu = args.cpu_sample or (160 if method == semb.CMP else 8)
        rate, secs, text = cpu_rate(oracle, s, method, cdp_end, n_cpu, seed=1, threads=threads)
        cpu = {"value": rate, "unit": "evals/s", "cores": threads, "kind": "port",
               "sample": f"{text}, {secs:.1f} s of CPU search (oracle restatement, OpenMP)"}

    peak = semb.probe_fp32_tflops(dev)
    traffic = traffic_from_profiles(args.workload, st["ncdps"], st["trace_evals"])
    hbm = None
    if traffic is not None:
        # HBM side of the roofline: DRAM bytes per launch over the live launch time,
        # against the measured copy bandwidth
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm_peak = float(json.load(f)["hbm_gbs"])
        except (OSError, ValueError, KeyError):
            hbm_peak = None
        got = traffic / (ms_search * 1e-3) / 1e9
        hbm = {"achieved_gbs": got, "peak_gbs": hbm_peak, "frac": got / hbm_peak if hbm_peak else None,
               "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy)"}
    roof = fp32_roofline(method, st, nap, ms_search, peak)
    roof.update({"traffic": traffic, "traffic_unit": "DRAM bytes per search launch (ncu)", "hbm": hbm,
                 "smem": smem_from_profiles(args.workload), "flops_per_launch": flops, "launch_ms": ms_search})
    clocks = clk.summary()
    cfg = workload_config(args.workload, s, method, world, nap / st["ncdps"])
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg, "store": args.storage, "graph": bool(args.graph),
            "plain_f32": res["plain"], "batched": res["batched"],
            "speedup_batched_vs_plain": res["plain"]["ms"] / (total_ms / args.steps),
            "roofline": roof, "clocks": clocks, "gpu_launches": int(st["kernel_launches"]) * args.steps,
            "autotune": {"variant": st["variant"], "sample_ms": tune[1] if tune else None,
                         "ctas_per_sm": st["ctas_per_sm"],
                         "buckets": [dict(zip(("ap_lo", "ap_hi", "tasks", "variant"), b)) for b in buckets]}}
    for k in ("store_bf16", "store_f32"):
        if k in res:
            line[k] = res[k]
    if e2e:
        line["e2e"] = e2e
    if err:
        line["error_vs_fp64"] = err
    if cpu:
        line["cpu_baseline"] = cpu
    plan.close()
    plain.close()
    pinned.free()
    if world == 1 and not args.no_target:
        line["target"] = run_target(args, dev)
    elif world > 1:
        line["target"] = {"skipped": "the 20k-CDP CRS goal is a one-GPU figure; measured by the N = 1 run"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="cmp-4096-uneven")
    ap.add_argument("--ncdp", type=int, default=None)
    ap.add_argument("--storage", choices=["f16", "bf16", "f32"], default=None)
    ap.add_argument("--graph", type=int, default=1)
    ap.add_argument("--tune", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--stream-chunks", type=int, default=16, help="CDP chunks of the streamed end-to-end run")
    ap.add_argument("--repick-gap", type=float, default=None,
                    help="near-tie threshold of the FP64 re-pick (default: the library's)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--variant", type=int, default=None, help="force this search-kernel variant (no autotuning)")
    ap.add_argument("--chunk-cdps", type=int, default=0,
                    help="instead of the benchmark line: one run of the whole workload in chunks of this many CDPs "
                         "(one CUDA graph per chunk) with FP64 errors on a sample")
    ap.add_argument("--err-frac", type=float, default=0.01, help="chunked run: fraction of CDPs in the error sample")
    ap.add_argument("--err-t0-blocks", type=int, default=1, help="chunked run: 32-sample t0 blocks per sampled CDP")
    ap.add_argument("--err-seed", type=int, default=17, help="chunked run: seed of the error sample")
    ap.add_argument("--no-target", action="store_true", help="skip the 20k-CDP CRS goal leg")
    ap.add_argument("--target-ncdp", type=int, default=None, help="CDPs of the goal leg's survey (default 20000)")
    ap.add_argument("--target-err-per-bucket", type=int, default=8,
                    help="CDPs per aperture bucket in the goal leg's FP64 error sample")
    ap.add_argument("--target-t0-blocks", type=int, default=4,
                    help="seeded 32-sample t0 blocks per CDP in the goal leg's FP64 error sample")
    args = ap.parse_args()
    if args.storage is None:
        args.storage = WORKLOAD_STORAGE.get(args.workload, "f16")
    if args.warmup < 3:
        log("warm-up raised to 3 steps (timing rule)")
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.gpus != world:
        log(f"--gpus {args.gpus} but WORLD_SIZE {world}: launch N > 1 with torchrun, one rank per GPU")
        return 2
    dist = None
    if world > 1:
        import torch.distributed as tdist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo", rank=rank, world_size=world)
        dist = tdist
    try:
        if args.impl == "reference":
            return run_reference_arm(args, rank, world)
        if args.chunk_cdps > 0:
            if world > 1:
                log("the chunked whole-survey run is a one-GPU run")
                return 2
            return run_chunked_survey(args)
        return run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
