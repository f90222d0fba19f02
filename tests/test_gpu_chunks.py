"""Chunked runs of the batched search (GPU): the survey searched in contiguous CDP
chunks, each chunk's work one CUDA graph captured on its first run and replayed
afterwards, gives exactly the unchunked results."""
import numpy as np
import pytest

import semb
import synth

pytestmark = pytest.mark.gpu


def _arrays(s):
    h = s.headers
    cdp_end = np.cumsum(s.info["fold"]).astype(np.int64)
    return semb.GatherArrays(cdp_end, s.ns, int(h["dt"][0]), h["gx"], h["gy"], h["sx"], h["sy"], h["scalco"],
                             s.samples)


def _surveys():
    # apertures 30-1500 traces: several aperture buckets, each with its own variant
    crs = synth.crs_survey(seed=81, ncdp=300, ns=200, dt_us=4000, na=3, nb=3, nc=3, tau=0.004, aph=2600, apm=150,
                           aperture_range=(30, 1500), block=8, line_len=300)
    cmp = synth.cmp_survey(seed=82, ncmp=90, ns=400, nc=40, tau=0.004, fold_range=(6, 120), hmax=2000.0, aph=2000)
    return [(semb.CRS, crs), (semb.CMP, cmp)]


@pytest.mark.parametrize("case", [0, 1])
def test_three_chunk_graphs_equal_the_unchunked_run(case):
    method, s = _surveys()[case]
    with semb.Plan(semb.params(method, mode=semb.BATCHED, **s.params)) as plan:
        plan.upload(_arrays(s).view())
        plan.autotune()
        plan.run()
        ref = plan.download()
        assert plan.chunk_times() == []
        per = (s.info["ncdp"] + 2) // 3
        plan.set_chunks(per)
        for rep in range(2):   # capture, then replay
            plan.run()
            out = plan.download()
            for a, b in zip(out, ref):
                assert np.array_equal(a, b), rep
            ms = plan.chunk_times()
            assert len(ms) == 3 and all(m > 0 for m in ms)
            assert plan.stats()["kernel_launches"] >= 3 * (2 if method == semb.CMP else 3)
        # back to one piece
        plan.set_chunks(0)
        plan.run()
        for a, b in zip(plan.download(), ref):
            assert np.array_equal(a, b)


def test_chunks_are_the_batched_grid_search():
    method, s = _surveys()[1]
    with semb.Plan(semb.params(method, mode=semb.PLAIN_F32, **s.params)) as plan:
        with pytest.raises(semb.SembError):
            plan.set_chunks(10)
