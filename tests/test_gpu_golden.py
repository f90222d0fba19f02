"""The CUDA path against the reference's own outputs (GPU), through the C ABI and
the command lines.

Plain form: semblance and stack within 1e-5 relative of the reference's
single-precision build, and identical picks wherever the best two semblances
(from the oracle's full table) differ by more than 1e-6.  Batched form: semblance
within 1e-3 absolute of the reference's double-precision build, at least 99.5%
identical picks, and 99.9% where the FP64 best two differ by more than 1e-6.
The command lines (plain form) match the reference build of their own precision
(FP32) and stay within a stated bound of the shipped CRS build (FP64)."""
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
import oracle
import semb

pytestmark = pytest.mark.gpu

METHOD = {"cmp": semb.CMP, "crs": semb.CRS}
BUILD = os.path.join(os.path.dirname(semb.LIB_PATH))


def _run_product(path, meta, **kw):
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    with semb.Plan(semb.params(METHOD[method], **p, **kw)) as plan:
        plan.upload(sv.view())
        plan.run()
        ctr, sem, stk = plan.download()
    return sv.arrays()["cdp"], ctr, sem, stk


def _top2_gap(meta, h, s):
    method, p = meta["method"], meta["params"]
    g = oracle.gather(h, s, method, p["aph"], p.get("apm"), real=np.float32)
    out = (oracle.cmp if method == "cmp" else oracle.crs)(g, p, "f32", sem_all=True)
    srt = np.sort(out["sem_all"], axis=2)
    return g["cdp_ids"], srt[:, :, -1] - srt[:, :, -2]


@pytest.mark.parametrize("case", G.CASES)
def test_plain_matches_reference_f32(case):
    meta, h, s, path = G.load(case)
    method = meta["method"]
    cdps, ctr, sem, stk = _run_product(path, meta, mode=semb.PLAIN_F32)
    ref = G.ref_outputs(case, method, "f32")
    rows = G.rows_by_cdp(cdps, ref["coher"][0])
    np.testing.assert_allclose(sem[rows], ref["coher"][1], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk[rows], ref["stack"][1], rtol=1e-5, atol=1e-6)
    gcdps, gap = _top2_gap(meta, h, s)
    decisive = gap[G.rows_by_cdp(gcdps, ref["coher"][0])] > 1e-6
    # the reference's picked parameter values, recomputed from our picks
    g = oracle.gather(h, s, method, meta["params"]["aph"], meta["params"].get("apm"), real=np.float32)
    o = (oracle.cmp if method == "cmp" else oracle.crs)(g, meta["params"], "f32")
    orow = G.rows_by_cdp(g["cdp_ids"], ref["coher"][0])
    assert np.array_equal(ctr[rows][decisive], o["ctr"][orow][decisive])
    assert np.array_equal(o["c"][orow], ref["c"][1])


@pytest.mark.parametrize("case", G.CASES)
def test_batched_close_to_reference_f64(case):
    meta, h, s, path = G.load(case)
    method = meta["method"]
    cdps, ctr, sem, stk = _run_product(path, meta, mode=semb.BATCHED)
    ref = G.ref_outputs(case, method, "f64")
    rows = G.rows_by_cdp(cdps, ref["coher"][0])
    assert np.max(np.abs(sem[rows] - ref["coher"][1])) <= 1e-3
    g = oracle.gather(h, s, method, meta["params"]["aph"], meta["params"].get("apm"), real=np.float64)
    o = (oracle.cmp if method == "cmp" else oracle.crs)(g, meta["params"], "f64", top2=True)
    orow = G.rows_by_cdp(g["cdp_ids"], ref["coher"][0])
    same = ctr[rows] == o["ctr"][orow]
    decisive = o["top2"][orow] > 1e-6
    assert same.mean() >= 0.995, same.mean()
    if decisive.any():
        assert same[decisive].mean() >= 0.999, same[decisive].mean()


@pytest.mark.parametrize("case", G.CASES)
def test_cli_end_to_end(case, tmp_path):
    """cmp-gb300 / crs-gb300 with the reference's flags write the reference's files:
    same headers and CDP order, semblance and stack within tolerance."""
    meta, h, s, path = G.load(case)
    method = meta["method"]
    exe = os.path.join(BUILD, f"{method}-gb300")
    r = subprocess.run([exe] + meta["args"] + ["-i", path, "-v", "2"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Execution Time" in r.stdout
    import su
    mine = {a: su.read_su(str(tmp_path / f"{method}.{a}.su")) for a in G.ATTRS[method]}
    shipped = {a: su.read_su(G.ref_file(case, method, G.SHIPPED[method], a)) for a in G.ATTRS[method]}
    for attr in G.ATTRS[method]:
        assert np.array_equal(mine[attr][0].view(np.uint8), shipped[attr][0].view(np.uint8)), attr
    # the command line searches in the plain form (FP32 arithmetic): against the
    # reference's FP32 build the files match within 1e-5 relative, with the same
    # picks where the best two differ by more than 1e-6
    ref32 = {a: su.read_su(G.ref_file(case, method, "f32", a)) for a in G.ATTRS[method]}
    np.testing.assert_allclose(mine["coher"][1], ref32["coher"][1], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(mine["stack"][1], ref32["stack"][1], rtol=1e-5, atol=1e-6)
    # the parameter files (c, or a, b, c) hold the picked candidate's value computed
    # in the shipped build's precision: equal to the shipped files wherever the pick
    # is decided (best two more than 1e-6 apart) and the FP32 and FP64 searches pick
    # alike
    gcdps, gap = _top2_gap(meta, h, s)
    orow = G.rows_by_cdp(gcdps, ref32["coher"][0])
    mask = gap[orow] > 1e-6
    if G.SHIPPED[method] == "f64":
        p = meta["params"]
        fn = oracle.cmp if method == "cmp" else oracle.crs
        o32 = fn(oracle.gather(h, s, method, p["aph"], p.get("apm"), real=np.float32), p, "f32")
        o64 = fn(oracle.gather(h, s, method, p["aph"], p.get("apm"), real=np.float64), p, "f64")
        mask &= (o32["ctr"] == o64["ctr"])[orow]
    for a in G.ATTRS[method][:-2]:
        assert np.array_equal(mine[a][1][mask], shipped[a][1][mask]), a
    # against the shipped CRS build (FP64): FP32 arithmetic stays within 1e-4 of the
    # FP64 coherence (the reference's own FP32 build is within 8.5e-5 of its FP64 build
    # on every golden case)
    np.testing.assert_allclose(mine["coher"][1], shipped["coher"][1], rtol=0, atol=1e-4)


@pytest.mark.parametrize("case", ["cmp_line", "crs_line"])
def test_cli_attribute_files(case, tmp_path):
    """-attrs 1 -mode batched also writes the aperture map, the second-best semblance
    and the FP64 error of the pick, one trace per CDP like the coherence file."""
    meta, h, s, path = G.load(case)
    method = meta["method"]
    exe = os.path.join(BUILD, f"{method}-gb300")
    r = subprocess.run([exe] + meta["args"] + ["-i", path, "-mode", "batched", "-attrs", "1"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    import su
    hc, coher = su.read_su(str(tmp_path / f"{method}.coher.su"))
    for name in ("aperture", "coher2", "err64"):
        hx, x = su.read_su(str(tmp_path / f"{method}.{name}.su"))
        assert hx.tobytes() == hc.tobytes() and x.shape == coher.shape, name
    _, ap = su.read_su(str(tmp_path / f"{method}.aperture.su"))
    assert np.all(ap >= 1) and np.all(ap == ap[:, :1])
    _, c2 = su.read_su(str(tmp_path / f"{method}.coher2.su"))
    assert np.all(c2 <= coher + 1e-3)


def test_graph_replay_matches_direct_launch():
    meta, h, s, path = G.load("crs_uneven_w5")
    p = meta["params"]
    sv = semb.Survey.load(path, semb.CRS, p["aph"])
    with semb.Plan(semb.params(semb.CRS, mode=semb.BATCHED, **p)) as plan:
        plan.upload(sv.view())
        plan.run()
        a = plan.download()
        plan.use_graph(True)
        plan.run()
        plan.run()
        b = plan.download()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("case", ["cmp_line", "crs_line"])
def test_autotuned_variants_agree(case):
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    with semb.Plan(semb.params(METHOD[method], mode=semb.BATCHED, **p)) as plan:
        plan.upload(sv.view())
        plan.run()
        base = plan.download()
        v, ms = plan.autotune()
        assert ms[v] > 0 and all(m < 0 or m >= ms[v] for m in ms)
        plan.run()
        tuned = plan.download()
        assert plan.stats()["variant"] == v
    assert np.mean(base[0] == tuned[0]) >= 0.999
    np.testing.assert_allclose(base[1], tuned[1], atol=1e-5)


def test_reupload_and_rerun_are_stable():
    meta, h, s, path = G.load("cmp_uneven_w1")
    p = meta["params"]
    sv = semb.Survey.load(path, semb.CMP, p["aph"])
    with semb.Plan(semb.params(semb.CMP, mode=semb.PLAIN_F32, **p)) as plan:
        outs = []
        for _ in range(2):
            plan.upload(sv.view())
            plan.run()
            plan.run()
            outs.append(plan.download())
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("mode", [semb.PLAIN_F32, semb.BATCHED])
def test_reupload_of_other_surveys_reuses_buffers_safely(mode):
    """One plan uploads a large, a small and the large survey again (the device
    buffers of the first are kept and reused): each result equals a fresh plan's."""
    meta_a, _, _, path_a = G.load("crs_uneven_w5")
    meta_b, _, _, path_b = G.load("crs_line")
    pa, pb = meta_a["params"], meta_b["params"]
    sva = semb.Survey.load(path_a, semb.CRS, pa["aph"])
    svb = semb.Survey.load(path_b, semb.CRS, pa["aph"])

    def fresh(sv):
        with semb.Plan(semb.params(semb.CRS, mode=mode, **pa)) as q:
            q.upload(sv.view())
            q.run()
            return q.download()

    ref_a, ref_b = fresh(sva), fresh(svb)
    with semb.Plan(semb.params(semb.CRS, mode=mode, **pa)) as plan:
        for sv, ref in ((sva, ref_a), (svb, ref_b), (sva, ref_a)):
            plan.upload(sv.view())
            plan.run()
            out = plan.download()
            for x, y in zip(out, ref):
                assert np.array_equal(x, y)


@pytest.mark.parametrize("case", ["cmp_uneven_w1", "crs_line", "crs_uneven_w5"])
@pytest.mark.parametrize("nchunks", [1, 3, 7])
def test_streamed_search_equals_upload_and_run(case, nchunks):
    """semb_plan_stream (chunked trace copies overlapped with the search of chunks
    whose apertures, halos included, have landed) gives the upload + run results."""
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    with semb.Plan(semb.params(METHOD[method], mode=semb.BATCHED, **p)) as plan:
        plan.upload(sv.view())
        plan.run()
        ref = plan.download()
        plan.stream(sv.view(), nchunks)
        out = plan.download()
        for x, y in zip(out, ref):
            assert np.array_equal(x, y)
        plan.run()   # the plan is uploaded afterwards
        for x, y in zip(plan.download(), ref):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("case", ["cmp_line", "cmp_uneven_w1", "cmp_farout", "crs_line", "crs_uneven_w5"])
def test_every_variant_agrees_with_the_default(case):
    """Each search-kernel variant (items per thread, CTAs per SM, staging and
    candidate layouts) gives the default variant's picks and semblances."""
    meta, h, s, path = G.load(case)
    method, p = meta["method"], meta["params"]
    sv = semb.Survey.load(path, METHOD[method], p["aph"])
    with semb.Plan(semb.params(METHOD[method], mode=semb.BATCHED, repick=semb.REPICK_OFF, **p)) as plan:
        plan.upload(sv.view())
        plan.run()
        base = plan.download()
        tried = 0
        for v in range(1, semb.MAX_VARIANTS):
            try:
                plan.set_variant(v)
            except semb.SembError:
                continue
            tried += 1
            plan.run()
            out = plan.download()
            assert np.mean(out[0] == base[0]) >= 0.995, v
            np.testing.assert_allclose(out[1], base[1], atol=2e-6, rtol=1e-5)
        assert tried >= 1
