"""The CUDA path against the oracle at the benchmark workloads' shapes (GPU).

The golden cases are small; these run the surveys the benchmark names, or seeded
samples of them, through the C ABI and check them against the oracle (the CPU
restatement of the reference's search, pinned bit for bit to the reference's own
programs):

* the 200-CMP line (60 traces, ns 1000, 101 velocities, w 3) in full;
* 32 CMPs of the uneven-fold line (fold 12-240, ns 2000, 256 velocities, w 5);
* 6 contiguous CDPs inside the 500-CDP CRS line (48 offsets, ns 1000, 21^3 grid),
  searched as part of the whole line;
* a CRS block shaped like the 20k-CDP survey (ns 1500 at 4 ms, 21^3 grid, tau 4 ms,
  apm 150 m, azimuth 90) whose apertures reach ~2,000 traces: every task then spans
  many staging chunks, both in-range and partly out-of-range traces, and the top-4
  lists merge over 83 candidate passes.

Plain form: semblance and stack within 1e-5 relative of the FP32 oracle and the
same picks wherever the oracle's best two semblances differ by more than 1e-6.
Batched form: semblance within 1e-3 of the FP64 oracle and at least 99.5% of the
picks identical to the FP64 oracle's, 99.9% where its best two differ by more than
1e-6.  Where a survey is too large for the CPU oracle in seconds, the oracle runs
on a seeded range of output samples (its t0 range) of some CDPs."""
import numpy as np
import pytest

import oracle
import semb
import synth

pytestmark = pytest.mark.gpu

SEM_TOL_BATCHED = 1e-3    # semblance, batched form vs FP64
PICKS_RAW = 0.995         # identical picks, batched form vs FP64
PICKS_DECISIVE = 0.999    # ... where the FP64 best two differ by more than 1e-6
TIE = 1e-6


def _arrays(g):
    return semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                             g["scalco"], g["samples"])


def _search(method, g, params, variant=None, **kw):
    with semb.Plan(semb.params(method, **params, **kw)) as p:
        p.upload(_arrays(g).view())
        if variant is not None:
            p.set_variant(variant)
        p.run()
        return p.download()


def _check_plain(out, ref, rows, t0s):
    ctr, sem, stk = (a[np.ix_(rows, t0s)] for a in out)
    np.testing.assert_allclose(sem, ref["str"][np.ix_(rows, t0s)], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk, ref["stk"][np.ix_(rows, t0s)], rtol=1e-5, atol=1e-6)
    decisive = ref["top2"][np.ix_(rows, t0s)] > TIE
    assert np.array_equal(ctr[decisive], ref["ctr"][np.ix_(rows, t0s)][decisive])


def _check_batched(out, ref64, rows, t0s):
    ctr, sem, stk = (a[np.ix_(rows, t0s)] for a in out)
    assert np.max(np.abs(sem - ref64["str"][np.ix_(rows, t0s)])) <= SEM_TOL_BATCHED
    same = ctr == ref64["ctr"][np.ix_(rows, t0s)]
    decisive = ref64["top2"][np.ix_(rows, t0s)] > TIE
    assert same.mean() >= PICKS_RAW, same.mean()
    if decisive.any():
        assert same[decisive].mean() >= PICKS_DECISIVE, same[decisive].mean()


def test_cmp_200x60_line_in_full():
    s = synth.config(0)
    g32 = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float32)
    g64 = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float64)
    rows, t0s = np.arange(len(g32["cdp_ids"])), np.arange(s.ns)
    _check_plain(_search(semb.CMP, g32, s.params, mode=semb.PLAIN_F32), oracle.cmp(g32, s.params, "f32", top2=True),
                 rows, t0s)
    _check_batched(_search(semb.CMP, g64, s.params, mode=semb.BATCHED), oracle.cmp(g64, s.params, "f64", top2=True),
                   rows, t0s)


def test_cmp_uneven_fold_sample_of_32():
    s = synth.config(1, ncdp=32)
    g32 = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float32)
    g64 = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float64)
    folds = np.diff(np.concatenate([[0], g32["ntraces_by_cdp_id"]]))
    assert folds.min() < 30 and folds.max() > 120   # the sample spans the fold range
    rows, t0s = np.arange(32), np.arange(s.ns)
    _check_plain(_search(semb.CMP, g32, s.params, mode=semb.PLAIN_F32), oracle.cmp(g32, s.params, "f32", top2=True),
                 rows, t0s)
    _check_batched(_search(semb.CMP, g64, s.params, mode=semb.BATCHED), oracle.cmp(g64, s.params, "f64", top2=True),
                   rows, t0s)


def test_crs_500x48_line_block_of_6():
    s = synth.config(2)
    g32 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    g64 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    rows = np.arange(247, 253)        # interior CDPs: full 9-CDP apertures
    t0s = np.arange(0, 500)           # t0 = 0 included (the stack of t0 without a pick)
    ref32 = oracle.crs(g32, s.params, "f32", cdps=rows, t0_range=(0, 500), top2=True)
    _check_plain(_search(semb.CRS, g32, s.params, mode=semb.PLAIN_F32), ref32, rows, t0s)
    ref64 = oracle.crs(g64, s.params, "f64", cdps=rows, t0_range=(0, 500), top2=True)
    _check_batched(_search(semb.CRS, g64, s.params, mode=semb.BATCHED), ref64, rows, t0s)


def test_crs_block_with_2000_trace_apertures():
    s = synth.crs_survey(seed=9, ncdp=64, ns=1500, dt_us=4000, nevents=6, tau=0.004, aph=2600, apm=150,
                         azimuth=90.0, aperture_range=(1900, 2000), block=32, name="crs-block-ap2000")
    g32 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    g64 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    folds = np.diff(np.concatenate([[0], g32["ntraces_by_cdp_id"]]))
    rows = np.array([16, 47])
    ap = [folds[g32["nbr"][g32["nbr_off"][i]:g32["nbr_off"][i + 1]]].sum() for i in rows]
    assert min(ap) >= 1900
    lo, hi = 560, 688
    t0s = np.arange(lo, hi)
    ref32 = oracle.crs(g32, s.params, "f32", cdps=rows, t0_range=(lo, hi), top2=True)
    _check_plain(_search(semb.CRS, g32, s.params, mode=semb.PLAIN_F32), ref32, rows, t0s)
    ref64 = oracle.crs(g64, s.params, "f64", cdps=rows, t0_range=(lo, hi), top2=True)
    _check_batched(_search(semb.CRS, g64, s.params, mode=semb.BATCHED), ref64, rows, t0s)


SHARED_CENTRAL = 30   # CRS variant sharing the central traces' sums over A and B


def _check_same_search(out, base):
    """Two batched searches that differ only in the order of their FP32 sums: the same
    picks but for near ties (which the re-pick may then settle the other way, moving
    the semblance by the size of the tie) and semblances within a few FP32 roundings."""
    assert np.mean(out[0] == base[0]) >= 0.999
    np.testing.assert_allclose(out[1], base[1], atol=2e-5, rtol=1e-4)


def test_crs_shared_central_traces_500x48_block():
    """The CRS variant that leaves each task's central traces (zero midpoint distance)
    out of the staged chunks and adds their sums, computed once per pass and C value,
    to every (A, B) item: at the 500-CDP line's shapes it meets the batched bars against
    the FP64 oracle and gives the default variant's results within float summation
    order."""
    s = synth.config(2)
    g64 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    rows = np.arange(247, 253)
    t0s = np.arange(0, 500)
    ref64 = oracle.crs(g64, s.params, "f64", cdps=rows, t0_range=(0, 500), top2=True)
    out = _search(semb.CRS, g64, s.params, variant=SHARED_CENTRAL, mode=semb.BATCHED)
    _check_batched(out, ref64, rows, t0s)
    base = _search(semb.CRS, g64, s.params, variant=13, mode=semb.BATCHED)
    _check_same_search(out, base)


def test_crs_shared_central_traces_2000_trace_block():
    """The same variant on a block shaped like the 20k-CDP survey with ~2,000-trace
    apertures (25 CDPs within apm, the central CDP's traces a 25th of each aperture):
    the default variant's results within float summation order, on every CDP and t0."""
    s = synth.crs_survey(seed=9, ncdp=64, ns=1500, dt_us=4000, nevents=6, tau=0.004, aph=2600, apm=150,
                         azimuth=90.0, aperture_range=(1900, 2000), block=32, name="crs-block-ap2000")
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    out = _search(semb.CRS, g, s.params, variant=SHARED_CENTRAL, mode=semb.BATCHED)
    base = _search(semb.CRS, g, s.params, variant=13, mode=semb.BATCHED)
    _check_same_search(out, base)


def test_crs_b_runs_of_8_on_a_31_value_b_axis():
    """nb = 31, the B axis of the 100,000-CDP survey's 31^3 grid: B runs of 8 pad each
    (A, C) group to 32 candidate slots where runs of 7 pad it to 35, so the plan starts
    on variant 33 (runs of 8, central traces' sums shared, 384 threads).  It and variant
    32 (runs of 8, 512 threads) meet the batched bars against the FP64 oracle and give
    variant 13's results (runs of 7) within float summation order."""
    s = synth.crs_survey(seed=41, ncdp=24, noffsets=16, ns=400, dt_us=4000, na=3, nb=31, nc=3, tau=0.004, apm=50)
    g64 = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
    rows, t0s = np.arange(9, 15), np.arange(0, 400)
    ref64 = oracle.crs(g64, s.params, "f64", cdps=rows, t0_range=(0, 400), top2=True)
    with semb.Plan(semb.params(semb.CRS, mode=semb.BATCHED, **s.params)) as p:
        p.upload(_arrays(g64).view())
        assert [b[3] for b in p.buckets()] == [33] * len(p.buckets())
    base = _search(semb.CRS, g64, s.params, variant=13, mode=semb.BATCHED)
    for v in (33, 32):
        out = _search(semb.CRS, g64, s.params, variant=v, mode=semb.BATCHED)
        _check_batched(out, ref64, rows, t0s)
        _check_same_search(out, base)
