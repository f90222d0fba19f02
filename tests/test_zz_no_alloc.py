"""The allocation-free neighbour-list entry point (GPU).

semb_neighbours_noalloc serves callers that cannot call cudaMalloc while they run
(device memory owned by another allocator, loops that forbid allocation after
start-up).  It must return exactly the lists the reference's rule gives and the
search plan builds for the same CDPs: checked against the oracle's lists, against
the plan's all-pairs and grid-search lists, on two calls in a row, across several
tiles of its single-block offset scan, at its 131,072-CDP limit, and for its two
errors (a list buffer that is too small, a survey above the limit).  This file is
collected last so a failure here comes after every other test has run."""
import time

import numpy as np
import pytest

import oracle
import semb
import synth

pytestmark = pytest.mark.gpu

LIMIT = 131072


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _plan_lists(g, params):
    arrays = semb.GatherArrays(g["ntraces_by_cdp_id"], g["ns"], g["dt_us"], g["gx"], g["gy"], g["sx"], g["sy"],
                               g["scalco"], g["samples"])
    with semb.Plan(semb.params(semb.CRS, **params)) as p:
        p.upload(arrays.view())
        return p.neighbours()


def _first_fields(g):
    first = np.concatenate([[0], g["ntraces_by_cdp_id"][:-1]]).astype(np.int64)
    return {k: np.ascontiguousarray(g[k][first], dtype=np.int32) for k in ("gx", "gy", "sx", "sy", "scalco")}


def _noalloc(torch, fields, apm, capacity=None, check=True):
    """One call on device buffers owned by torch; returns (status, off, list)."""
    dev = {k: torch.from_numpy(v).cuda() for k, v in fields.items()}
    ncdp = len(fields["gx"])
    off = torch.full((ncdp + 1,), -5, dtype=torch.int32, device="cuda")
    cap = capacity if capacity is not None else 16 * ncdp
    lst = torch.full((max(cap, 1),), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc, n = semb.neighbours_noalloc(dev["gx"].data_ptr(), dev["gy"].data_ptr(), dev["sx"].data_ptr(),
                                    dev["sy"].data_ptr(), dev["scalco"].data_ptr(), ncdp, apm, off.data_ptr(),
                                    lst.data_ptr(), cap, stream, check=False)
    if check:
        assert rc == semb.OK, semb.lib().semb_last_error().decode()
    return rc, n, off.cpu().numpy(), lst.cpu().numpy()


def _line_lists(mx, my, apm):
    """The reference's rule (CRS/OpenMP/src/su_gather.cpp:70-87) for CDPs on a line
    with increasing midpoints: j is a neighbour of i when the float32 squared
    distance of their first-trace midpoints is within apm^2; lists ascending."""
    n = len(mx)
    lim = np.float32(apm * apm)
    step = float(np.min(np.abs(np.diff(mx.astype(np.float64))))) if n > 1 else 1.0
    K = int(np.ceil(apm / max(step, 1e-6))) + 2
    hits = []
    for d in range(-K, K + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        j = i + d
        dx = mx[j] - mx[i]
        dy = my[j] - my[i]
        ok = (dx * dx + dy * dy) <= lim
        hits.append(np.stack([i[ok], j[ok]], axis=1))
    pairs = np.concatenate(hits)
    pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, pairs[:, 0] + 1, 1)
    return np.cumsum(off).astype(np.int32), pairs[:, 1].astype(np.int32)


def test_noalloc_neighbours_match_plan_twice(torch):
    """Two calls in a row, on different surveys, each against the plan's lists."""
    for seed, ncdp, apm in ((31, 120, 50), (32, 75, 37)):
        s = synth.crs_survey(seed=seed, ncdp=ncdp, noffsets=4, ns=64, na=2, nb=2, nc=2, apm=apm)
        g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
        off_plan, lst_plan = _plan_lists(g, s.params)
        _, n, off_na, lst_na = _noalloc(torch, _first_fields(g), s.params["apm"])
        assert np.array_equal(off_na, off_plan)
        assert np.array_equal(lst_na[:n], lst_plan)


def test_noalloc_several_scan_tiles_match_oracle(torch):
    """1,500 CDPs: the per-CDP counts span two 1,024-entry tiles of the offset scan;
    the lists equal the oracle's restatement of the reference's neighbour rule."""
    s = synth.crs_survey(seed=33, ncdp=1500, noffsets=2, ns=32, na=1, nb=1, nc=1, apm=40, line_len=600)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    _, n, off, lst = _noalloc(torch, _first_fields(g), s.params["apm"])
    assert n == int(g["nbr_off"][-1])
    assert np.array_equal(off, g["nbr_off"])
    assert np.array_equal(lst[:n], g["nbr"])


def test_noalloc_matches_the_plans_grid_search(torch):
    """2,500 CDPs, where the plan builds its lists with the grid search instead of
    all pairs: the allocation-free lists are the same."""
    s = synth.crs_survey(seed=34, ncdp=2500, noffsets=2, ns=32, na=1, nb=1, nc=1, apm=30, line_len=500)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    off_plan, lst_plan = _plan_lists(g, s.params)
    _, n, off, lst = _noalloc(torch, _first_fields(g), s.params["apm"])
    assert np.array_equal(off, off_plan)
    assert np.array_equal(lst[:n], lst_plan)
    assert np.array_equal(off, g["nbr_off"]) and np.array_equal(lst[:n], g["nbr"])


def test_noalloc_small_buffer_reports_the_length(torch):
    """A list buffer below the total: SEMB_E_ARG, *n_list still gives the length
    needed, and nothing is written past the buffer."""
    s = synth.crs_survey(seed=35, ncdp=200, noffsets=2, ns=32, na=1, nb=1, nc=1, apm=50)
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    need = int(g["nbr_off"][-1])
    cap = need // 2
    rc, n, off, lst = _noalloc(torch, _first_fields(g), s.params["apm"], capacity=cap, check=False)
    assert rc == semb.E_ARG and n == need
    assert np.array_equal(off, g["nbr_off"])
    assert np.array_equal(lst[:cap], g["nbr"][:cap])


def test_noalloc_at_and_above_the_limit(torch):
    """131,072 CDPs on a line (the largest survey the fixed scratch holds) gives the
    reference rule's lists; one CDP more is SEMB_E_ARG before any device work."""
    n = LIMIT
    x_cm = (100000 + 1000 * np.arange(n)).astype(np.int64)   # 10 m apart
    fields = {"gx": (x_cm + 2500).astype(np.int32), "sx": (x_cm - 2500).astype(np.int32),
              "gy": np.zeros(n, np.int32), "sy": np.zeros(n, np.int32), "scalco": np.full(n, -100, np.int32)}
    fs = oracle.fscalco(fields["scalco"])
    mx = (fs * (fields["gx"] + fields["sx"]).astype(np.float32)) * np.float32(0.5)
    my = (fs * (fields["gy"] + fields["sy"]).astype(np.float32)) * np.float32(0.5)
    want_off, want = _line_lists(mx, my, 25)
    t0 = time.perf_counter()
    _, got_n, off, lst = _noalloc(torch, fields, 25, capacity=len(want) + 64)
    secs = time.perf_counter() - t0
    print(f"semb_neighbours_noalloc at {n} CDPs: {secs * 1e3:.1f} ms (host wall, incl. buffer set-up)")
    assert got_n == len(want)
    assert np.array_equal(off, want_off)
    assert np.array_equal(lst[:got_n], want)
    small = {k: v[:4].copy() for k, v in fields.items()}
    dev = {k: torch.from_numpy(v).cuda() for k, v in small.items()}
    out = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc, _ = semb.neighbours_noalloc(dev["gx"].data_ptr(), dev["gy"].data_ptr(), dev["sx"].data_ptr(),
                                    dev["sy"].data_ptr(), dev["scalco"].data_ptr(), n + 1, 25, out.data_ptr(),
                                    out.data_ptr(), 8, None, check=False)
    assert rc == semb.E_ARG
    assert "131072" in semb.lib().semb_last_error().decode()
