"""Aperture buckets of the batched work queue (GPU): each bucket has its own tuned
variant (neighbours on the same variant run as one launch), and the result does not
depend on how the queue is split."""
import numpy as np
import pytest

import semb
import synth

pytestmark = pytest.mark.gpu


def _survey():
    # apertures 30-1500 traces in blocks of 8 CDPs: several aperture buckets
    return synth.crs_survey(seed=31, ncdp=640, ns=200, dt_us=4000, na=3, nb=3, nc=3, tau=0.004, aph=2600,
                            apm=150, aperture_range=(30, 1500), block=8, line_len=640)


def _arrays(s):
    h = s.headers
    cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
    return semb.GatherArrays(cdp_end, s.ns, int(h["dt"][0]), h["gx"], h["gy"], h["sx"], h["sy"], h["scalco"],
                             s.samples)


def test_buckets_cover_the_queue_and_tuning_keeps_the_result():
    s = _survey()
    arrays = _arrays(s)
    nblk = (s.ns + 31) // 32
    with semb.Plan(semb.params(semb.CRS, mode=semb.BATCHED, repick=semb.REPICK_OFF, **s.params)) as plan:
        plan.upload(arrays.view())
        bs = plan.buckets()
        assert 2 <= len(bs) <= semb.MAX_BUCKETS
        assert sum(b[2] for b in bs) == len(s.info["fold"]) * nblk
        for (lo, hi, n, v), nxt in zip(bs, bs[1:] + [None]):
            assert lo <= hi and n > 0 and v >= 0
            if nxt is not None:
                assert nxt[1] <= lo   # sorted by decreasing aperture, no overlap
        plan.run()
        base = plan.download()
        chosen, ms = plan.autotune()
        assert chosen in [b[3] for b in plan.buckets()]
        assert ms[chosen] > 0
        tuned = plan.buckets()
        assert sum(b[2] for b in tuned) == len(s.info["fold"]) * nblk
        # neighbours with the same variant were merged
        assert all(a[3] != b[3] for a, b in zip(tuned, tuned[1:]))
        plan.run()
        out = plan.download()
        assert np.mean(out[0] == base[0]) >= 0.995
        np.testing.assert_allclose(out[1], base[1], atol=2e-6, rtol=1e-5)
        # one variant everywhere: every bucket runs it, all in one launch (stack of
        # t0 = 0 + search + re-pick)
        plan.set_variant(0)
        assert all(b[3] == 0 for b in plan.buckets())
        plan.run()
        assert plan.stats()["kernel_launches"] == 3
        out0 = plan.download()
        assert np.mean(out0[0] == base[0]) >= 0.995


def test_plain_form_is_one_bucket():
    s = _survey()
    with semb.Plan(semb.params(semb.CRS, mode=semb.PLAIN_F32, **s.params)) as plan:
        plan.upload(_arrays(s).view())
        bs = plan.buckets()
        assert len(bs) == 1 and bs[0][2] == len(s.info["fold"]) * ((s.ns + 31) // 32)
