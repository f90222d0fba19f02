"""CUDA path vs the oracle, through the C ABI (GPU)."""
import numpy as np
import pytest

import oracle
import semb
import synth

pytestmark = pytest.mark.gpu


def _arrays(g):
    return semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                             g["scalco"], g["samples"])


def _run(method, g, params, **kw):
    with semb.Plan(semb.params(method, **params, **kw)) as p:
        p.upload(_arrays(g).view())
        p.run()
        out = p.download()
        st = p.stats()
    return out, st


@pytest.mark.parametrize("ns,fold,nc,tau", [(400, 24, 33, 0.002), (500, 30, 101, 0.004), (300, 7, 16, 0.0)])
def test_cmp_plain_matches_oracle_f32(ns, fold, nc, tau):
    s = synth.cmp_survey(seed=21, ncmp=10, fold=fold, ns=ns, nc=nc, tau=tau)
    g = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"])
    ref = oracle.cmp(g, s.params, "f32")
    (ctr, sem, stk), _ = _run(semb.CMP, g, s.params, mode=semb.PLAIN_F32)
    assert np.array_equal(ctr, ref["ctr"])
    np.testing.assert_allclose(sem, ref["str"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk, ref["stk"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("na,nb,nc,tau", [(5, 5, 5, 0.002), (3, 4, 7, 0.004), (2, 1, 3, 0.0)])
def test_crs_plain_matches_oracle_f32(na, nb, nc, tau):
    s = synth.crs_survey(seed=22, ncdp=12, noffsets=16, ns=300, na=na, nb=nb, nc=nc, tau=tau)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    ref = oracle.crs(g, s.params, "f32")
    (ctr, sem, stk), _ = _run(semb.CRS, g, s.params, mode=semb.PLAIN_F32)
    assert np.array_equal(ctr, ref["ctr"])
    np.testing.assert_allclose(sem, ref["str"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk, ref["stk"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("storage", [semb.STORE_F16, semb.STORE_BF16, semb.STORE_F32])
def test_crs_batched_close_to_oracle_f64(storage):
    s = synth.crs_survey(seed=23, ncdp=12, noffsets=16, ns=300, na=5, nb=5, nc=5)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    ref = oracle.crs(g, s.params, "f64")
    (ctr, sem, stk), st = _run(semb.CRS, g, s.params, mode=semb.BATCHED, storage=storage)
    tol = 5e-3 if storage == semb.STORE_BF16 else 1e-3
    assert np.max(np.abs(sem - ref["str"])) < tol
    assert np.mean(ctr == ref["ctr"]) >= 0.995


def test_cmp_batched_close_to_oracle_f64():
    s = synth.cmp_survey(seed=24, ncmp=10, fold=24, ns=400, nc=33)
    g = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float64)
    ref = oracle.cmp(g, s.params, "f64")
    (ctr, sem, stk), st = _run(semb.CMP, g, s.params, mode=semb.BATCHED)
    assert np.max(np.abs(sem - ref["str"])) < 1e-3
    assert np.mean(ctr == ref["ctr"]) >= 0.995


def test_crs_neighbour_lists_match_reference_rule():
    s = synth.crs_survey(seed=25, ncdp=30, noffsets=6, ns=200, na=2, nb=2, nc=2)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    with semb.Plan(semb.params(semb.CRS, **s.params)) as p:
        p.upload(_arrays(g).view())
        off, lst = p.neighbours()
    assert np.array_equal(off, g["nbr_off"])
    assert np.array_equal(lst, g["nbr"])


def test_bounded_wait_gives_up_and_device_stays_usable():
    """A barrier nothing completes: the wait the search kernels use for their bulk
    copies gives up after its limit, and the GPU keeps working afterwards."""
    assert semb.selftest_wait(0, 20000) == 1
    s = synth.cmp_survey(seed=26, ncmp=3, fold=6, ns=200, nc=8)
    g = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"])
    (ctr, sem, stk), _ = _run(semb.CMP, g, s.params, mode=semb.PLAIN_F32)
    ref = oracle.cmp(g, s.params, "f32")
    assert np.array_equal(ctr, ref["ctr"])


@pytest.mark.parametrize("azimuth", [30.0, 90.0])
def test_crs_signed_dm_plain_matches_oracle_f32(azimuth):
    """SEMB_DM_SIGNED (dm projected on the azimuth, signed): the plain form against
    the oracle's signed branch in single precision."""
    s = synth.crs_survey(seed=42, ncdp=12, noffsets=16, ns=300, na=5, nb=3, nc=4, tau=0.004, azimuth=azimuth)
    p = dict(s.params)
    g = oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float32)
    ref = oracle.crs(g, p, "f32", dm_signed=True)
    (ctr, sem, stk), _ = _run(semb.CRS, g, p, mode=semb.PLAIN_F32, dm_mode=semb.DM_SIGNED)
    assert np.array_equal(ctr, ref["ctr"])
    np.testing.assert_allclose(sem, ref["str"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk, ref["stk"], rtol=1e-5, atol=1e-6)


def test_crs_signed_dm_batched_close_to_oracle_f64():
    s = synth.crs_survey(seed=43, ncdp=12, noffsets=16, ns=300, na=5, nb=5, nc=5, azimuth=30.0)
    p = dict(s.params)
    g = oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float64)
    ref = oracle.crs(g, p, "f64", dm_signed=True)
    (ctr, sem, stk), _ = _run(semb.CRS, g, p, mode=semb.BATCHED, dm_mode=semb.DM_SIGNED)
    assert np.max(np.abs(sem - ref["str"])) < 1e-3
    assert np.mean(ctr == ref["ctr"]) >= 0.995
    # and it is not the |dm| result
    absr = oracle.crs(g, p, "f64")
    assert not np.allclose(absr["str"], ref["str"])


def test_attribute_outputs():
    """Extra attributes: the aperture map, the second-best candidate and the FP64
    error of the pick (every (CDP, t0) re-evaluated with repick = ALWAYS)."""
    s = synth.crs_survey(seed=44, ncdp=12, noffsets=16, ns=300, na=5, nb=5, nc=5)
    p = dict(s.params)
    g = oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float64)
    ref = oracle.crs(g, p, "f64")
    folds = np.diff(np.concatenate([[0], g["ntraces_by_cdp_id"]]))
    ap_ref = np.array([folds[g["nbr"][g["nbr_off"][i]:g["nbr_off"][i + 1]]].sum() for i in range(len(folds))])
    with semb.Plan(semb.params(semb.CRS, mode=semb.BATCHED, repick=semb.REPICK_ALWAYS, attrs=1, **p)) as plan:
        plan.upload(_arrays(g).view())
        plan.run()
        ctr, sem, stk = plan.download()
        at = plan.download_attrs()
    assert np.array_equal(at["aperture"], ap_ref)
    picked = sem > 0
    # the FP64 error of every pick is known, small, and the pick's value is the FP64 one
    assert np.all(at["err64"][picked] >= 0) and np.max(at["err64"][picked]) < 1e-3
    np.testing.assert_allclose(sem[picked], ref["str"][picked], rtol=1e-6, atol=1e-7)
    # second best: another candidate, not better than the pick beyond FP32 error
    has2 = at["idx2"] >= 0
    assert np.mean(has2[picked]) > 0.9
    assert np.all(at["idx2"][has2] != ctr[has2])
    assert np.all(at["sem2"][has2] <= sem[has2] + 1e-3)
    # a plain plan has the aperture map only
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, **p)) as plain:
        plain.upload(_arrays(g).view())
        assert np.array_equal(plain.download_attrs(batched=False)["aperture"], ap_ref)
        with pytest.raises(semb.SembError):
            plain.download_attrs()


def test_grid_neighbour_lists_match_the_reference_rule():
    """Surveys of 2048 CDPs or more get their CRS neighbour lists from the grid
    search (cells + sorts); they equal the reference's all-pairs lists.  A 3D layout
    (a 55 x 55 grid of CDPs, 10 m apart, apm 25 m) has neighbours along x and y."""
    import su
    n1, ns = 55, 32
    ix, iy = np.meshgrid(np.arange(n1), np.arange(n1), indexing="ij")
    h = su.empty_headers(n1 * n1)
    h["cdp"] = np.arange(1, n1 * n1 + 1)
    h["scalco"] = -100
    # midpoints on the grid (cm), half-offset 50 m along x, with a little jitter
    rng = np.random.default_rng(46)
    mx = (ix.ravel() * 1000 + rng.integers(-40, 40, n1 * n1)).astype(np.int32)
    my = (iy.ravel() * 1000 + rng.integers(-40, 40, n1 * n1)).astype(np.int32)
    h["sx"], h["gx"], h["sy"], h["gy"] = mx - 5000, mx + 5000, my, my
    h["ns"], h["dt"] = ns, 4000
    samples = rng.standard_normal((n1 * n1, ns)).astype(np.float32)
    p = dict(a0=-1e-3, a1=1e-3, na=1, b0=0.0, b1=0.0, nb=1, c0=2e-7, c1=1e-6, nc=1, aph=100, apm=25, tau=0.0)
    g = oracle.gather(h, samples, "crs", p["aph"], p["apm"], real=np.float32)
    assert len(g["cdp_ids"]) >= 2048
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, **p)) as plan:
        plan.upload(_arrays(g).view())
        off, lst = plan.neighbours()
    assert np.array_equal(off, g["nbr_off"])
    assert np.array_equal(lst, g["nbr"])
    assert np.max(np.diff(off)) >= 9   # neighbours along x and y
