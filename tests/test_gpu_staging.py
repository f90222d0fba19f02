"""Staging capacity of the batched form (GPU).

The batched kernels stage each trace's window (the samples any item of a candidate
pass can read) in shared memory; a window longer than the stage is read from the
FP32 store in global memory instead, with the same arithmetic.  These surveys have
windows of hundreds to over a thousand samples (a pass spans the whole velocity or
C range at offsets up to 3 km), and the plans are forced to stages of 64-256
samples, so most far-offset traces take the global path.  With FP32 storage the
staged entries hold exactly the FP32 samples, so the results equal the default
staging's up to the order of the FP32 sums (smaller stages cut a pass into more
chunks, and a chunk's in-range traces are summed before its others); with FP16
storage they must stay within the batched form's error of the FP64 oracle."""
import numpy as np
import pytest

import oracle
import semb
import synth

pytestmark = pytest.mark.gpu


def _arrays(g):
    return semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                             g["scalco"], g["samples"])


def _surveys():
    cmp = synth.cmp_survey(seed=71, ncmp=6, ns=2000, dt_us=2000, nc=48, tau=0.004, fold_range=(20, 40), hmax=3000.0,
                           aph=3000)
    crs = synth.crs_survey(seed=72, ncdp=8, noffsets=24, ns=1500, dt_us=4000, na=2, nb=1, nc=40, tau=0.004,
                           aph=2600, apm=50)
    return [("cmp", semb.CMP, cmp), ("crs", semb.CRS, crs)]


def _gather(kind, s, real=np.float32):
    return oracle.gather(s.headers, s.samples, kind, s.params["aph"], s.params.get("apm"), real=real)


@pytest.mark.parametrize("case", [0, 1])
def test_small_stages_match_the_default_staging_with_fp32_storage(case):
    kind, method, s = _surveys()[case]
    g = _gather(kind, s)
    with semb.Plan(semb.params(method, mode=semb.BATCHED, storage=semb.STORE_F32, repick=semb.REPICK_OFF,
                               **s.params)) as plan:
        plan.upload(_arrays(g).view())
        variants = [v for v in range(semb.MAX_VARIANTS) if _has(plan, v)]
        assert variants
        for v in variants:
            plan.set_variant(v)
            plan.set_staging(0)
            plan.run()
            ref = plan.download()
            for cap in (256, 64):
                plan.set_staging(cap)
                plan.run()
                ctr, sem, stk = plan.download()
                assert np.mean(ctr == ref[0]) >= 0.999, (v, cap)
                np.testing.assert_allclose(sem, ref[1], rtol=1e-5, atol=1e-6, err_msg=f"{v} {cap}")
                np.testing.assert_allclose(stk, ref[2], rtol=1e-5, atol=1e-6, err_msg=f"{v} {cap}")


def _has(plan, v):
    try:
        plan.set_variant(v)
        return True
    except semb.SembError:
        return False


@pytest.mark.parametrize("case", [0, 1])
def test_small_stages_with_fp16_storage_stay_close_to_fp64(case):
    kind, method, s = _surveys()[case]
    g = _gather(kind, s, np.float64)
    ref = (oracle.cmp if method == semb.CMP else oracle.crs)(g, s.params, "f64", top2=True)
    with semb.Plan(semb.params(method, mode=semb.BATCHED, **s.params)) as plan:
        plan.upload(_arrays(g).view())
        plan.set_staging(128)
        plan.run()
        ctr, sem, stk = plan.download()
    assert np.max(np.abs(sem - ref["str"])) <= 1e-3
    same = ctr == ref["ctr"]
    assert same.mean() >= 0.995
    decisive = ref["top2"] > 1e-6
    assert same[decisive].mean() >= 0.999


def test_staging_capacity_is_checked():
    kind, method, s = _surveys()[1]
    with semb.Plan(semb.params(method, mode=semb.BATCHED, **s.params)) as plan:
        with pytest.raises(semb.SembError):
            plan.set_staging(10)
