"""The oracle (CPU restatement) pinned to the reference's own programs (CPU).

Against the golden files every output value must be bit-identical; where the
reference programs were built here (oracle/_ref), also on a fresh seeded case."""
import os
import tempfile

import numpy as np
import pytest

import golden_cases as G
import oracle
import synth


def _oracle_outputs(meta, h, s, prec):
    method, p = meta["method"], meta["params"]
    real = np.float32 if prec == "f32" else np.float64
    g = oracle.gather(h, s, method, p["aph"], p.get("apm"), real=real)
    out = oracle.cmp(g, p, prec) if method == "cmp" else oracle.crs(g, p, prec)
    vals = {"coher": out["str"].astype(np.float32), "stack": out["stk"].astype(np.float32), "c": out["c"]}
    if method == "crs":
        vals["a"], vals["b"] = out["a"], out["b"]
    return g, vals


@pytest.mark.parametrize("case", G.CASES)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_restatement_matches_reference_golden(case, prec):
    meta, h, s, _ = G.load(case)
    g, vals = _oracle_outputs(meta, h, s, prec)
    ref = G.ref_outputs(case, meta["method"], prec)
    for attr, (rh, rd) in ref.items():
        rows = G.rows_by_cdp(g["cdp_ids"], rh)
        assert np.array_equal(vals[attr][rows].view(np.uint32), rd.view(np.uint32)), (case, prec, attr)


def test_golden_cases_cover_edge_cases():
    names = set(G.CASES)
    assert {"cmp_line", "cmp_uneven_w1", "cmp_farout", "crs_line", "crs_uneven_w5"} <= names
    # the far-offset case has traces out of the record, so invalid (-1) semblances
    # and t0 with no pick exist
    meta, h, s, _ = G.load("cmp_farout")
    c = G.ref_outputs("cmp_farout", "cmp", "f32")["c"][1]
    assert np.any(c == 0.0) and np.any(c > 0.0)


@pytest.mark.skipif(not oracle.have_reference(), reason="reference programs not built here")
@pytest.mark.parametrize("method", ["cmp", "crs"])
def test_restatement_matches_reference_live(method):
    if method == "cmp":
        sv = synth.cmp_survey(seed=202, ncmp=18, fold=9, ns=150, nc=20, tau=0.002)
    else:
        sv = synth.crs_survey(seed=203, ncdp=9, noffsets=5, ns=120, na=3, nb=2, nc=3, tau=0.004, apm=40)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.su")
        sv.write(path)
        meta = {"method": method, "params": sv.params}
        for prec in ("f32", "f64"):
            ref = oracle.run_reference(method, prec, path, sv.cli_args("x")[:-2], workdir=d)
            g, vals = _oracle_outputs(meta, sv.headers, sv.samples, prec)
            for attr in G.ATTRS[method]:
                rh, rd = ref[attr]
                rows = G.rows_by_cdp(g["cdp_ids"], rh)
                assert np.array_equal(vals[attr][rows].view(np.uint32), rd.view(np.uint32)), (method, prec, attr)
