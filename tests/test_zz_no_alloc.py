"""The allocation-free neighbour-list entry point against the plan's lists (GPU).

semb_neighbours_noalloc serves callers that cannot call cudaMalloc while they run;
it must return exactly the lists the search plan builds for the same CDPs.  This
file is collected last so a failure here comes after every other test has run."""
import numpy as np
import pytest

import oracle
import semb
import synth

pytestmark = pytest.mark.gpu


def _plan_lists(g, params):
    arrays = semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                               g["scalco"], g["samples"])
    with semb.Plan(semb.params(semb.CRS, **params)) as p:
        p.upload(arrays.view())
        return p.neighbours()


def _noalloc_lists(g, apm, torch):
    first = np.concatenate([[0], g["ntraces_by_cdp_id"][:-1]]).astype(np.int64)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a[first], dtype=np.int32)).cuda()
    gx, gy, sx, sy, sc = (dev(g[k]) for k in ("gx", "gy", "sx", "sy", "scalco"))
    ncdp = len(first)
    off = torch.zeros(ncdp + 1, dtype=torch.int32, device="cuda")
    cap = ncdp * ncdp
    lst = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    n = semb.neighbours_noalloc(gx.data_ptr(), gy.data_ptr(), sx.data_ptr(), sy.data_ptr(), sc.data_ptr(), ncdp, apm,
                                off.data_ptr(), lst.data_ptr(), cap, stream)
    return off.cpu().numpy(), lst[:n].cpu().numpy()


def test_noalloc_neighbours_match_plan_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # two calls in a row, on different surveys, each against the plan's lists
    for seed, ncdp, apm in ((31, 120, 50), (32, 75, 37)):
        s = synth.crs_survey(seed=seed, ncdp=ncdp, noffsets=4, ns=64, na=2, nb=2, nc=2, apm=apm)
        g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
        off_plan, lst_plan = _plan_lists(g, s.params)
        off_na, lst_na = _noalloc_lists(g, s.params["apm"], torch)
        assert np.array_equal(off_na, off_plan)
        assert np.array_equal(lst_na, lst_plan)
