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

--impl reference times the reference's own CPU implementation of the path instead
(oracle/_ref when it was built on this machine, else the oracle restatement).
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

def make_gather(name: str, ncdp: int | None):
    """Synthetic survey of a workload; traces are CDP-major, so cdp_end follows
    from the folds.  Every rank gets the same workload (weak scaling)."""
    idx, n_default, method = WORKLOADS[name]
    s = synth.config(idx, ncdp=ncdp or n_default)
    cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
    return s, method, cdp_end, s.headers


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

def algo_flops(method: int, st: dict, nap: int) -> float:
    """Algorithmic FLOPs of one search: per eval N_ap*(T + 7w) + 2w + 2 with T = 5
    (CMP: add, mul, sqrt, scale, frac) or 10 (CRS), per window sample 3 for the
    interpolation, 1 for num, 2 for den, 1 for lin."""
    w = st["window"]
    T = 5 if method == semb.CMP else 10
    per_cand_t0 = nap * (T + 7 * w) + st["ncdps"] * (2 * w + 2)
    return float(st["ns"]) * st["ncand"] * per_cand_t0


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


def subset(s, cdp_end, idx):
    """Headers/samples of the CDPs in idx (a gather restricted to them)."""
    starts = np.concatenate([[0], cdp_end[:-1]])
    rows = np.concatenate([np.arange(starts[i], cdp_end[i]) for i in idx])
    return s.headers[rows], s.samples[rows]


_GATHERS = {}


def _full_gather(oracle, s, precision):
    key = (id(s), precision)
    if key not in _GATHERS:
        _GATHERS[key] = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"],
                                      real=np.float32 if precision == "f32" else np.float64)
    return _GATHERS[key]


def cpu_rate(oracle, s, method, cdp_end, n_sample, seed, precision="f32", threads=0):
    """Oracle on a seeded sample of CDPs; returns (evals/s, seconds, sample text)."""
    ncdp = len(cdp_end)
    rng = np.random.default_rng(seed)
    if method == semb.CMP:
        idx = np.sort(rng.choice(ncdp, size=min(n_sample, ncdp), replace=False))
        h, d = subset(s, cdp_end, idx)
        g = oracle.gather(h, d, "cmp", s.params["aph"], real=np.float32 if precision == "f32" else np.float64)
        out = oracle.cmp(g, s.params, precision, threads=threads)
        ncand = int(s.params["nc"])
        text = f"{len(idx)} seeded-random CMPs of {ncdp}"
    else:
        # CRS apertures span neighbouring CDPs: search the sample inside the whole gather
        start = int(rng.integers(0, max(1, ncdp - n_sample)))
        idx = np.arange(start, min(ncdp, start + n_sample))
        g = _full_gather(oracle, s, precision)
        out = oracle.crs(g, s.params, precision, threads=threads, cdps=idx)
        ncand = int(s.params["na"]) * int(s.params["nb"]) * int(s.params["nc"])
        text = f"{len(idx)} contiguous CDPs of {ncdp}"
    evals = len(idx) * s.ns * ncand
    return evals / out["seconds"], out["seconds"], text, idx, out, g


# ----------------------------------------------------------------------------- arms

def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    s, method, cdp_end, _ = make_gather(args.workload, args.ncdp)
    oracle = oracle_mod()
    threads = os.cpu_count() or 1
    n_sample = args.cpu_sample or (96 if method == semb.CMP else 2)
    kind = "port"
    vals = []
    for step in range(args.warmup + args.steps):
        rate, secs, text, *_ = cpu_rate(oracle, s, method, cdp_end, n_sample, seed=step, threads=threads)
        if step >= args.warmup:
            vals.append(rate)
    value = statistics.median(vals)
    ms = s.ns * n_sample * (int(s.params["nc"]) if method == semb.CMP else
                            int(s.params["na"]) * int(s.params["nb"]) * int(s.params["nc"])) / value * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "sample_per_step": text},
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": kind,
                             "sample": text + " per step (CPU restatement of the reference's OpenMP search)"},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, world, dist):
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    t_gen = time.perf_counter()
    s, method, cdp_end, _ = make_gather(args.workload, args.ncdp)
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
    tune = plan.autotune() if args.tune else None
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

    # error of the batched form against the FP64 oracle on a sample
    err = None
    cpu = None
    if rank == 0 and not args.no_cpu:
        oracle = oracle_mod()
        ctr_b, sem_b, stk_b = plan.download()
        ctr_p, sem_p, stk_p = plain.download()
        n_err = 24 if method == semb.CMP else 2
        _, secs64, text64, idx, o64, _ = cpu_rate(oracle, s, method, cdp_end, n_err, seed=7, precision="f64")
        rows = idx
        if method == semb.CMP:
            sem64, pick64, stk64 = o64["str"], o64["ctr"], o64["stk"]
        else:
            sem64, pick64, stk64 = o64["str"][rows], o64["ctr"][rows], o64["stk"][rows]
        # near-tie-free picks: FP64 top-two gap above 1e-6 needs the full table; report raw identity
        err = {"sample": text64 + " (FP64 oracle)",
               "batched_sem_max_abs": float(np.max(np.abs(sem_b[rows] - sem64))),
               "batched_stack_max_abs": float(np.max(np.abs(stk_b[rows] - stk64))),
               "batched_identical_picks": float(np.mean(ctr_b[rows] == pick64)),
               "plain_sem_max_abs": float(np.max(np.abs(sem_p[rows] - sem64))),
               "plain_identical_picks": float(np.mean(ctr_p[rows] == pick64))}
        threads = os.cpu_count() or 1
        n_cpu = args.cpu_sample or (160 if method == semb.CMP else 2)
        rate, secs, text, *_ = cpu_rate(oracle, s, method, cdp_end, n_cpu, seed=1, threads=threads)
        cpu = {"value": rate, "unit": "evals/s", "cores": threads, "kind": "port",
               "sample": f"{text}, {secs:.1f} s of CPU search (oracle restatement, OpenMP)"}

    peak = semb.probe_fp32_tflops(dev)
    achieved = flops / (ms_search * 1e-3) / 1e12
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
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic, "traffic_unit": "DRAM bytes per search launch (ncu)", "hbm": hbm,
            "smem": smem_from_profiles(args.workload),
            "peak_source": "measured live: semb_probe_fp32 FMA throughput",
            "flops_per_launch": flops, "launch_ms": ms_search}
    clocks = clk.summary()
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "name": s.name, "storage": args.storage, "ncdps": st["ncdps"],
                       "ns": st["ns"], "ncand": st["ncand"], "window": st["window"], "traces": s.ntraces,
                       "mean_aperture": nap / st["ncdps"], "trace_evals_per_step": st["trace_evals"],
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (%s store %.2f GB)" % (
                           args.storage.upper(), s.samples.nbytes / (1e9 if args.storage == "f32" else 2e9)),
                       "graph": bool(args.graph)},
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.close()
    plain.close()
    pinned.free()
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
    ap.add_argument("--stream-chunks", type=int, default=8, help="CDP chunks of the streamed end-to-end run")
    ap.add_argument("--repick-gap", type=float, default=None,
                    help="near-tie threshold of the FP64 re-pick (default: the library's)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true")
    args = ap.parse_args()
    if args.storage is None:
        args.storage = WORKLOAD_STORAGE.get(args.workload, "f16")
    if args.warmup < 3:
        log("warm-up raised to 3 steps (timing rule)")
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo", rank=rank, world_size=world)
        dist = tdist
    try:
        if args.impl == "reference":
            return run_reference_arm(args, rank, world)
        return run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
