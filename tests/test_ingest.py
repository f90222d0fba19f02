"""Host side of the product (CPU): SU ingest, CDP grouping and order, the output
writer, and error handling, through the C ABI."""
import os
import tempfile

import numpy as np
import pytest

import golden_cases as G
import oracle
import semb
import su

METHOD = {"cmp": semb.CMP, "crs": semb.CRS}


@pytest.mark.parametrize("case", G.CASES)
def test_survey_grouping_matches_oracle(case, semb_lib):
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    a = sv.arrays()
    g = oracle.gather(h, s, method, p["aph"], p.get("apm"), real=np.float32 if method == "cmp" else np.float64)
    assert sorted(a["cdp"].tolist()) == sorted(g["cdp_ids"].tolist())
    assert a["ns"] == g["ns"] and a["dt_us"] == g["dt_us"]
    starts = np.concatenate([[0], a["cdp_end"][:-1]])
    gstarts = np.concatenate([[0], g["ntraces_by_cdp_id"][:-1]])
    for i, c in enumerate(a["cdp"]):
        j = int(np.nonzero(g["cdp_ids"] == c)[0][0])
        sl, gl = slice(starts[i], a["cdp_end"][i]), slice(gstarts[j], g["ntraces_by_cdp_id"][j])
        assert np.array_equal(a["samples"][sl], g["samples"][gl])
        for k in ("gx", "gy", "sx", "sy", "scalco"):
            assert np.array_equal(a[k][sl], g[k][gl])
    if method == "cmp":
        # CMPs ordered by decreasing fold
        folds = np.diff(np.concatenate([[0], a["cdp_end"]]))
        assert np.all(np.diff(folds) <= 0)


@pytest.mark.parametrize("case", [c for c in G.CASES if c.startswith("cmp")])
def test_cmp_output_order_matches_reference(case, semb_lib):
    meta, h, s, path = G.load(case)
    sv = semb.Survey.load(path, semb.CMP, meta["params"]["aph"])
    rh, _ = G.ref_outputs(case, "cmp", "f32")["coher"]
    assert sv.arrays()["cdp"].tolist() == rh["cdp"].tolist()


@pytest.mark.parametrize("case", G.CASES)
def test_writer_reproduces_reference_files(case, semb_lib):
    """Fed the reference's own results, the writer produces the reference's files
    byte for byte (headers, CDP order, attribute values)."""
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    prec = G.SHIPPED[method]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    a = sv.arrays()
    g = oracle.gather(h, s, method, p["aph"], p.get("apm"), real=np.float32 if method == "cmp" else np.float64)
    out = oracle.cmp(g, p, prec) if method == "cmp" else oracle.crs(g, p, prec)
    rows = G.rows_by_cdp(g["cdp_ids"], {"cdp": a["cdp"]})
    ctr = out["ctr"][rows]
    sem = out["str"][rows].astype(np.float32)
    stk = out["stk"][rows].astype(np.float32)
    params = semb.params(METHOD[method], **p)
    with tempfile.TemporaryDirectory() as d:
        sv.write(params, ctr, sem, stk, d)
        for attr in G.ATTRS[method]:
            with open(os.path.join(d, f"{method}.{attr}.su"), "rb") as f1, \
                    open(G.ref_file(case, method, prec, attr), "rb") as f2:
                assert f1.read() == f2.read(), (case, attr)


def test_truncated_trace_is_a_format_error(semb_lib, tmp_path):
    meta, h, s, path = G.load("cmp_line")
    data = open(path, "rb").read()
    bad = tmp_path / "bad.su"
    bad.write_bytes(data[:-10])
    with pytest.raises(semb.SembError) as e:
        semb.Survey.load(str(bad), semb.CMP, 800)
    assert e.value.code == semb.E_FORMAT


def test_short_header_at_end_is_ignored(semb_lib, tmp_path):
    meta, h, s, path = G.load("cmp_line")
    data = open(path, "rb").read()
    f = tmp_path / "tail.su"
    f.write_bytes(data + b"\0" * 100)
    a = semb.Survey.load(str(f), semb.CMP, 800).arrays()
    b = semb.Survey.load(path, semb.CMP, 800).arrays()
    assert np.array_equal(a["samples"], b["samples"])


def test_mixed_ns_is_a_format_error(semb_lib, tmp_path):
    hdr = su.empty_headers(2)
    hdr["cdp"] = 1
    hdr["dt"] = 2000
    hdr["ns"] = [10, 12]
    rec = hdr[0].tobytes() + np.zeros(10, np.float32).tobytes() + hdr[1].tobytes() + np.zeros(12, np.float32).tobytes()
    with pytest.raises(semb.SembError) as e:
        semb.Survey.from_bytes(rec, semb.CMP, 100)
    assert e.value.code == semb.E_FORMAT


def test_missing_file_is_an_io_error(semb_lib):
    with pytest.raises(semb.SembError) as e:
        semb.Survey.load("/nonexistent/x.su", semb.CRS, 100)
    assert e.value.code == semb.E_IO


def test_offset_aperture_filter(semb_lib):
    """Traces whose half-offset exceeds aph are dropped; the boundary is kept."""
    meta, h, s, path = G.load("cmp_line")
    data = open(path, "rb").read()
    hx = np.abs(h["gx"].astype(np.int64) - h["sx"]) / 100.0 / 2.0
    for aph in (0, int(np.median(hx)), int(hx.max())):
        a = semb.Survey.load(path, semb.CMP, aph).arrays()
        assert a["ntraces"] == int(np.sum(hx <= aph))


@pytest.mark.parametrize("case", ["cmp_line", "crs_line"])
def test_attribute_writer(case, semb_lib):
    """semb_survey_write_attr: one trace per CDP in the survey's order, the CDP's first
    trace header unchanged (as the coherence file), the given samples."""
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    a = sv.arrays()
    ncdp, ns = len(a["cdp"]), a["ns"]
    data = np.arange(ncdp * ns, dtype=np.float32).reshape(ncdp, ns) * np.float32(0.5)
    ctr = np.zeros((ncdp, ns), np.int32)
    sem = np.zeros((ncdp, ns), np.float32)
    with tempfile.TemporaryDirectory() as d:
        sv.write(semb.params(METHOD[method], **p), ctr, sem, sem, d)
        sv.write_attr(f"{method}.extra.su", data, d)
        hx, sx = su.read_su(os.path.join(d, f"{method}.extra.su"))
        hc, _ = su.read_su(os.path.join(d, f"{method}.coher.su"))
    assert np.array_equal(sx, data)
    assert hx.tobytes() == hc.tobytes()


def test_explicit_parameter_writer_matches_the_grid_writer(semb_lib):
    """semb_survey_write_abc (CRS-DE outputs) writes the same five files, with the same
    headers, as the grid-search writer; the samples are the given A, B, C (C back in the
    reference's unscaled units is the caller's), coherence and stack."""
    meta, h, s, path = G.load("crs_line")
    p = meta["params"]
    sv = semb.Survey.load(path, semb.CRS, p["aph"])
    a = sv.arrays()
    ncdp, ns = len(a["cdp"]), a["ns"]
    rng = np.random.default_rng(3)
    vals = [rng.standard_normal((ncdp, ns)).astype(np.float32) for _ in range(5)]
    ctr = np.zeros((ncdp, ns), np.int32)
    with tempfile.TemporaryDirectory() as d1, tempfile.TemporaryDirectory() as d2:
        sv.write(semb.params(semb.CRS, **p), ctr, vals[3], vals[4], d1)
        sv.write_abc(*vals, d2)
        for k, name in enumerate(("a", "b", "c", "coher", "stack")):
            h1, _ = su.read_su(os.path.join(d1, f"crs.{name}.su"))
            h2, x2 = su.read_su(os.path.join(d2, f"crs.{name}.su"))
            assert h1.tobytes() == h2.tobytes(), name
            assert np.array_equal(x2, vals[k]), name
    with pytest.raises(semb.SembError):
        semb.Survey.load(G.load("cmp_line")[3], semb.CMP, 800).write_abc(*vals, ".")
