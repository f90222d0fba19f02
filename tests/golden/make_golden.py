"""Generate the golden fixtures in this directory (run where the reference tree is).

    python tests/golden/make_golden.py [case ...]     (default: every case)

Writes small seeded SU inputs and the outputs of the reference's own OpenMP
programs on them, built from the reference sources by oracle/Makefile (make ref):
cmp-omp2 (single precision, as shipped) and cmp-omp2-fp64, crs-omp2 (double, as
shipped) and crs-omp2-fp32.  Each case is a directory <case>/ with in.su, args.json
and <binary>/<method>.<attr>.su.  The tests compare the oracle restatement and the
CUDA path against these files, so the pin also holds where the reference is absent.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ipdps-crs-cmp-code_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
import synth  # noqa: E402


def cases():
    """(name, survey) pairs: small versions of the workloads plus edge cases."""
    out = []
    # 20 equal-fold CMPs: exercises the reference's unstable fold sort (more than 16
    # elements) and the CMP output order
    out.append(("cmp_line", synth.cmp_survey(seed=101, ncmp=20, fold=8, ns=256, dt_us=4000, nc=16, tau=0.008,
                                             half_offsets=25.0 + 50.0 * np.arange(8))))
    # uneven folds, w = 1 (tau below dt), positive scalco, one all-zero trace
    s = synth.cmp_survey(seed=102, ncmp=12, ns=200, dt_us=4000, nc=12, tau=0.002, fold_range=(3, 14), hmax=400.0)
    s.headers["scalco"] = 1
    for k in ("sx", "sy", "gx", "gy"):
        s.headers[k] = np.rint(s.headers[k] / 100.0).astype(np.int32)
    s.samples[5, :] = 0.0
    out.append(("cmp_uneven_w1", s))
    # long offsets: traces running out of the record (one out of range still counts,
    # two make the item invalid: -1 semblances and t0 without a pick)
    out.append(("cmp_farout", synth.cmp_survey(seed=103, ncmp=6, fold=10, ns=150, dt_us=4000, nc=10, tau=0.004,
                                               half_offsets=50.0 + 100.0 * np.arange(10), aph=3000)))
    # CRS line, zero scalco, w = 3
    s = synth.crs_survey(seed=104, ncdp=10, noffsets=6, ns=200, dt_us=4000, na=3, nb=3, nc=3, tau=0.004)
    s.headers["scalco"] = 0
    for k in ("sx", "sy", "gx", "gy"):
        s.headers[k] = np.rint(s.headers[k] / 100.0).astype(np.int32)
    out.append(("crs_line", s))
    # CRS along y (azimuth 90), uneven apertures, w = 5
    out.append(("crs_uneven_w5", synth.crs_survey(seed=105, ncdp=14, ns=200, dt_us=4000, na=2, nb=3, nc=4,
                                                  tau=0.008, aph=500, apm=60, azimuth=90.0,
                                                  aperture_range=(6, 40), block=4, line_len=7)))
    # CMP at the largest window the reference allows (tau = 7 samples, w = 15 < MAX_W = 16)
    out.append(("cmp_wmax", synth.cmp_survey(seed=106, ncmp=8, fold=12, ns=300, dt_us=4000, nc=12, tau=0.028)))
    # tiny gathers: CMPs of two or three traces (w = 5 at 2 ms, 64 velocities), where
    # near-tied velocities are resolved by few samples
    out.append(("cmp_tiny", synth.cmp_survey(seed=107, ncmp=24, ns=500, dt_us=2000, nc=64, tau=0.004,
                                             fold_range=(2, 3), hmax=1500.0, aph=1500)))
    # CRS apertures of two traces of one CDP (CDPs farther apart than apm): dm = 0, so
    # A and B do not change the traveltime and candidates tie exactly
    out.append(("crs_tiny", synth.crs_survey(seed=108, ncdp=12, noffsets=2, ns=300, dt_us=4000, na=3, nb=3, nc=8,
                                             tau=0.004, spacing=200.0, apm=50, aph=600)))
    return out


def main():
    if not oracle.have_reference():
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    only = set(sys.argv[1:])
    for name, s in cases():
        if only and name not in only:
            continue
        d = os.path.join(HERE, name)
        shutil.rmtree(d, ignore_errors=True)
        os.makedirs(d)
        s.write(os.path.join(d, "in.su"))
        args = s.cli_args("in.su")[:-2]
        with open(os.path.join(d, "args.json"), "w") as f:
            json.dump({"method": s.method, "args": args, "params": {k: (float(v) if isinstance(v, float) else v)
                                                                    for k, v in s.params.items()}}, f, indent=1)
        for prec in ("f32", "f64"):
            exe = os.path.basename(oracle.ref_binary(s.method, prec))
            od = os.path.join(d, exe)
            os.makedirs(od)
            out = oracle.run_reference(s.method, prec, os.path.join(d, "in.su"), args, workdir=od)
            with open(os.path.join(od, "info.txt"), "w") as f:
                f.write(out["info"].split(": ", 2)[-1] + "\n")
        print(name, s.ntraces, "traces")


if __name__ == "__main__":
    main()
