"""CRS-DE restatement (CPU): properties of the differential-evolution search that
the GPU path is checked against.  The reference's crs-ocl-de source is not in the
reference, so the method is the library's definition (semb_oracle_body.h)."""
import numpy as np

import oracle
import synth


def _case():
    s = synth.crs_survey(seed=51, ncdp=4, noffsets=8, ns=120, dt_us=4000, na=4, nb=3, nc=4, tau=0.004)
    p = dict(s.params)
    return p, oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float32)


def test_zero_generations_is_the_grid_search():
    p, g = _case()
    grid = oracle.crs(g, p, "f32")
    de = oracle.crs_de(g, p, 0, "f32")
    assert np.array_equal(de["str"], grid["str"])
    assert np.array_equal(de["stk"], grid["stk"])
    for k in ("a", "b", "c"):
        assert np.array_equal(de[k], grid[k]), k


def test_evolution_never_loses_the_best_and_is_reproducible():
    p, g = _case()
    grid = oracle.crs(g, p, "f32")
    de = oracle.crs_de(g, p, 12, "f32")
    assert np.all(de["str"] >= grid["str"])      # selection keeps every individual's best
    assert np.mean(de["str"] > grid["str"]) > 0.2
    again = oracle.crs_de(g, p, 12, "f32", threads=2)
    assert np.array_equal(again["str"], de["str"]) and np.array_equal(again["c"], de["c"])
    # parameters stay inside the search box
    assert np.all((de["a"] >= np.float32(p["a0"])) & (de["a"] <= np.float32(p["a1"])))
    assert np.all((de["c"] >= np.float32(p["c0"]) * 0.999) & (de["c"] <= np.float32(p["c1"]) * 1.001))
