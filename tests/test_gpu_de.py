"""CRS-DE on the GPU (differential evolution over A, B, C; -ngen): the same picks,
semblances and stacks as the oracle's restatement in single precision, bit for bit."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import semb
import su
import synth

pytestmark = pytest.mark.gpu

BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ipdps-crs-cmp-code_gb300", "_build")


def _arrays(g):
    return semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                             g["scalco"], g["samples"])


def _case(seed=61, **kw):
    s = synth.crs_survey(seed=seed, ncdp=8, noffsets=10, ns=200, dt_us=4000, na=5, nb=4, nc=5, tau=0.004, **kw)
    p = dict(s.params)
    return s, p, oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float32)


def test_zero_generations_is_the_grid_search():
    """ngen = 0 is the plan's grid search, whose picks the DE restatement reproduces
    from its starting population."""
    s, p, g = _case()
    ref = oracle.crs_de(g, p, 0, "f32")
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, **p)) as plan:
        plan.upload(_arrays(g).view())
        plan.run()
        ctr, sem, stk = plan.download()
    assert np.all(ctr >= 0)
    np.testing.assert_allclose(sem, ref["str"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(stk, ref["stk"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("ngen", [1, 15])
def test_de_matches_oracle_f32(ngen):
    s, p, g = _case()
    ref = oracle.crs_de(g, p, ngen, "f32")
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, ngen=ngen, **p)) as plan:
        plan.upload(_arrays(g).view())
        plan.run()
        ctr, sem, stk = plan.download()
        a, b, c = plan.download_abc()
    assert np.all(ctr == -1)
    assert np.array_equal(sem, ref["str"])
    assert np.array_equal(stk, ref["stk"])
    assert np.array_equal(a, ref["a"]) and np.array_equal(b, ref["b"]) and np.array_equal(c, ref["c"])


def test_de_signed_dm_and_grid_plan_has_no_abc():
    s, p, g = _case(seed=62, azimuth=30.0)
    ref = oracle.crs_de(g, p, 8, "f32", dm_signed=True)
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, ngen=8, dm_mode=semb.DM_SIGNED, **p)) as plan:
        plan.upload(_arrays(g).view())
        plan.run()
        _, sem, _ = plan.download()
    assert np.array_equal(sem, ref["str"])
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, **p)) as grid:
        grid.upload(_arrays(g).view())
        grid.run()
        with pytest.raises(semb.SembError):
            grid.download_abc()
    with pytest.raises(semb.SembError):
        semb.Plan(semb.params(semb.CRS, mode=semb.BATCHED, ngen=8, **p))


def test_cli_ngen_writes_the_crs_files(tmp_path):
    s, p, g = _case(seed=63)
    path = str(tmp_path / "in.su")
    s.write(path)
    args = s.cli_args("in.su")[:-2]
    r = subprocess.run([os.path.join(BUILD, "crs-gb300")] + args + ["-i", path, "-ngen", "10"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = oracle.crs_de(g, p, 10, "f32")
    _, coher = su.read_su(str(tmp_path / "crs.coher.su"))
    _, cval = su.read_su(str(tmp_path / "crs.c.su"))
    assert np.array_equal(coher, ref["str"]) and np.array_equal(cval, ref["c"])
