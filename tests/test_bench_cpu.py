"""bench.py on the CPU: the reference arm's JSON line (the oracle restatement timed on
the host cores) and the DRAM-traffic figures it takes from the ncu summaries."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench  # noqa: E402
    return bench


def test_reference_arm_prints_one_contract_line():
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build")):
        pytest.skip("oracle not built (build() compiles it)")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "cmp-4096-uneven", "--ncdp", "48", "--steps", "1", "--warmup", "3", "--cpu-sample", "4"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == _bench().METRIC and d["unit"] == "evals/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["value"] == d["value"]
    # the same workload description as the GPU arm's line
    for k in ("workload", "name", "ncdps", "ns", "ncand", "window", "traces", "mean_aperture", "parallelism"):
        assert k in d["config"], k
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_traffic_from_profiles_scales_by_trace_evaluations():
    bench = _bench()
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        table = json.load(f)
    src = table["crs-uneven-2000"]
    captured = src["dram_read"] + src["dram_write"]
    # the captured case itself
    assert bench.traffic_from_profiles("crs-uneven-2000", src["ncdps"], src["trace_evals"]) == captured
    # another CDP count of the same workload, and the 20k survey scaled from it
    assert bench.traffic_from_profiles("crs-uneven-2000", 1000, src["trace_evals"] // 2) == pytest.approx(captured / 2)
    assert bench.traffic_from_profiles("crs-uneven-20k", 20000, 10 * src["trace_evals"]) == pytest.approx(10 * captured)
    assert bench.traffic_from_profiles("no-such-workload", 1, 1) is None
    smem = bench.smem_from_profiles("crs-uneven-20k")
    assert 0 < smem["load_wavefronts_pct_of_peak"] <= 100 and smem["source"].startswith("ncu")


def test_reference_arm_under_torchrun_prints_from_rank_0_only():
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build")):
        pytest.skip("oracle not built (build() compiles it)")
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--gpus", "2", "--impl", "reference", "--workload", "cmp-4096-uneven", "--ncdp", "48",
                        "--steps", "1", "--warmup", "3", "--cpu-sample", "4"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
