"""The oracle's sampling options (CPU): a t0 range evaluates the same values as the
full search on those rows, and the top-2 gap equals the one taken from the full
candidate table.  The bench and the GPU parity tests at the benchmark shapes use
them to check large surveys on a sample of output samples."""
import numpy as np
import pytest

import oracle
import synth


@pytest.mark.parametrize("method", ["cmp", "crs"])
def test_t0_range_and_top2_match_the_full_search(method):
    if method == "cmp":
        s = synth.cmp_survey(seed=61, ncmp=5, fold=12, ns=300, nc=24, tau=0.004)
        g = oracle.gather(s.headers, s.samples, "cmp", s.params["aph"], real=np.float64)
        run = lambda **kw: oracle.cmp(g, s.params, "f64", **kw)
    else:
        s = synth.crs_survey(seed=62, ncdp=8, noffsets=8, ns=240, na=3, nb=3, nc=4, tau=0.004)
        g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float64)
        run = lambda **kw: oracle.crs(g, s.params, "f64", **kw)
    full = run(sem_all=True)
    lo, hi = 37, 181
    part = run(t0_range=(lo, hi), top2=True, cdps=[1, 3, 4])
    for k in ("ctr", "str", "stk"):
        assert np.array_equal(part[k][[1, 3, 4], lo:hi], full[k][[1, 3, 4], lo:hi]), k
    assert not np.any(part["str"][:, :lo]) and not np.any(part["str"][:, hi:])
    srt = np.sort(full["sem_all"], axis=2)
    gap = srt[:, :, -1] - srt[:, :, -2]
    assert np.array_equal(part["top2"][[1, 3, 4], lo:hi], gap[[1, 3, 4], lo:hi])
    assert np.all(np.isnan(part["top2"][0])) and np.all(np.isnan(part["top2"][:, :lo]))
    # settings do not leak into the next search
    again = run()
    assert np.array_equal(again["str"], full["str"])
