"""The bounds-checked build (GPU): libsemb_gb300_checked.so runs the same searches
with every staged-window read tested against the window the planner staged for its
trace.  On the golden cases (every kernel variant, both forms), the benchmark-shaped
surveys and plans with stages smaller than a trace, no check may fire, and the
results must be the production library's.  The checked library runs in a child
process (SEMB_CHECKED=1 selects it when the binding loads)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import golden_cases as G
import semb
import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r'''
import json, sys
import numpy as np
import golden_cases as G, semb, synth
assert semb.LIB_PATH.endswith("libsemb_gb300_checked.so"), semb.LIB_PATH
out = {}
M = {"cmp": semb.CMP, "crs": semb.CRS}

def run(tag, method, params, view, variant=None, staging=None, **kw):
    with semb.Plan(semb.params(method, **params, **kw)) as p:
        p.upload(view)
        if variant is not None:
            p.set_variant(variant)
        if staging is not None:
            p.set_staging(staging)
        p.run()
        c, s, k = p.download()
    out[tag] = [c.tolist(), s.tolist(), k.tolist()]

for case in G.CASES:
    meta, h, s, path = G.load(case)
    sv = semb.Survey.load(path, M[meta["method"]], meta["params"]["aph"])
    run(case + "/plain", M[meta["method"]], meta["params"], sv.view(), mode=semb.PLAIN_F32)
    for v in range(semb.MAX_VARIANTS):
        try:
            run(case + f"/v{v}", M[meta["method"]], meta["params"], sv.view(), variant=v, mode=semb.BATCHED)
        except semb.SembError as e:
            if e.code == semb.E_BOUNDS:
                raise
s = synth.crs_survey(seed=9, ncdp=64, ns=1500, dt_us=4000, nevents=6, tau=0.004, aph=2600, apm=150,
                     azimuth=90.0, aperture_range=(1900, 2000), block=32)
h = s.headers
cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
arr = semb.GatherArrays(cdp_end, s.ns, int(h["dt"][0]), h["gx"], h["gy"], h["sx"], h["sy"], h["scalco"], s.samples)
run("crs-ap2000/batched", semb.CRS, s.params, arr.view(), mode=semb.BATCHED)
run("crs-ap2000/staging128", semb.CRS, s.params, arr.view(), staging=128, mode=semb.BATCHED)
s = synth.config(1, ncdp=32)
h = s.headers
cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
arr = semb.GatherArrays(cdp_end, s.ns, int(h["dt"][0]), h["gx"], h["gy"], h["sx"], h["sy"], h["scalco"], s.samples)
run("cmp-uneven32/batched", semb.CMP, s.params, arr.view(), mode=semb.BATCHED)
run("cmp-uneven32/plain", semb.CMP, s.params, arr.view(), mode=semb.PLAIN_F32)
json.dump(out, open(sys.argv[1], "w"))
'''


def test_checked_build_finds_no_window_outside_its_staging(tmp_path):
    lib = os.path.join(ROOT, "ipdps-crs-cmp-code_gb300", "_build", "libsemb_gb300_checked.so")
    assert os.path.exists(lib), "build() makes the checked library"
    res = tmp_path / "checked.json"
    env = dict(os.environ, SEMB_CHECKED="1",
               PYTHONPATH=os.pathsep.join([HERE, os.path.join(ROOT, "ipdps-crs-cmp-code_gb300"),
                                           os.path.join(ROOT, "oracle")]))
    r = subprocess.run([sys.executable, "-c", CHILD, str(res)], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    got = json.loads(res.read_text())
    assert len(got) > 2 * len(G.CASES)
    # the production library computes the same results
    M = {"cmp": semb.CMP, "crs": semb.CRS}
    for case in G.CASES:
        meta, h, s, path = G.load(case)
        sv = semb.Survey.load(path, M[meta["method"]], meta["params"]["aph"])
        with semb.Plan(semb.params(M[meta["method"]], mode=semb.PLAIN_F32, **meta["params"])) as p:
            p.upload(sv.view())
            p.run()
            ref = p.download()
        for a, b in zip(got[case + "/plain"], ref):
            assert np.array_equal(np.asarray(a, dtype=b.dtype), b), case
