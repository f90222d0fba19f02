"""Multi-process sharding (CPU, gloo, world sizes 2 and 3).

Each rank owns a contiguous CDP range and loads, read-only, the halo CDPs within
apm; the CRS search of its owned CDPs must then equal the single-process search.
The search here is the oracle, standing in for the GPU on a CPU-only machine; what
is under test is the host logic that decides which traces a rank needs."""
import os
import socket

import numpy as np
import pytest

import oracle
import shard
import synth


def _survey():
    return synth.crs_survey(seed=41, ncdp=24, noffsets=4, ns=96, dt_us=4000, na=2, nb=2, nc=3, tau=0.004,
                            apm=40, spacing=12.5)


def _rank_result(rank, world):
    s = _survey()
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    first = np.concatenate([[0], g["ntraces_by_cdp_id"][:-1]])
    first_hdr = {k: g[k][first] for k in ("gx", "gy", "sx", "sy", "scalco")}
    cdp_end = g["ntraces_by_cdp_id"].astype(np.int64)
    sh = shard.plan_shard("crs", cdp_end, first_hdr, s.params["apm"], world, rank)
    part = sh.select(cdp_end, {k: g[k] for k in ("gx", "gy", "sx", "sy", "scalco", "samples")})
    local = dict(part, ntraces_by_cdp_id=part["cdp_end"].astype(np.int32), ns=g["ns"], dt_us=g["dt_us"],
                 cdp_ids=g["cdp_ids"][sh.cdps])
    # neighbour lists inside the shard
    lf = np.concatenate([[0], local["ntraces_by_cdp_id"][:-1]])
    mx, my = shard.first_trace_midpoints({k: local[k][lf] for k in ("gx", "gy", "sx", "sy", "scalco")})
    lists = shard.neighbours_of(mx, my, s.params["apm"], range(len(sh.cdps)))
    local["nbr_off"] = np.concatenate([[0], np.cumsum([len(x) for x in lists])]).astype(np.int32)
    local["nbr"] = np.concatenate(lists).astype(np.int32)
    out = oracle.crs(local, s.params, "f32", cdps=sh.owned_local, threads=1)
    return sh.owned, out["str"][sh.owned_local], out["ctr"][sh.owned_local], out["stk"][sh.owned_local]


def _worker(rank, world, port, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    res = _rank_result(rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    if rank == 0:
        np.save(result_path, np.array(gathered, dtype=object), allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_split_ranges_balance_and_cover():
    w = np.array([5, 1, 1, 1, 5, 1, 1, 1, 1, 5], float)
    for world in (1, 2, 3, 4):
        r = shard.split_ranges(w, world)
        assert r[0][0] == 0 and r[-1][1] == len(w)
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))


def test_halo_holds_every_neighbour_of_the_owned_cdps():
    s = _survey()
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    first = np.concatenate([[0], g["ntraces_by_cdp_id"][:-1]])
    first_hdr = {k: g[k][first] for k in ("gx", "gy", "sx", "sy", "scalco")}
    cdp_end = g["ntraces_by_cdp_id"].astype(np.int64)
    mx, my = shard.first_trace_midpoints(first_hdr)
    for world in (1, 2, 3, 5):
        owned_all = []
        for rank in range(world):
            sh = shard.plan_shard("crs", cdp_end, first_hdr, s.params["apm"], world, rank)
            lo, hi = sh.owned
            owned_all.extend(range(lo, hi))
            assert np.array_equal(sh.cdps[sh.owned_local], np.arange(lo, hi))
            for nb in shard.neighbours_of(mx, my, s.params["apm"], range(lo, hi)):
                assert np.isin(nb, sh.cdps).all()
        assert owned_all == list(range(len(cdp_end)))


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_reproduce_single_process_search(tmp_path, world):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    path = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(world, _free_port(), path), nprocs=world, join=True, start_method="spawn")
    gathered = np.load(path, allow_pickle=True)
    s = _survey()
    g = oracle.gather(s.headers, s.samples, "crs", s.params["aph"], s.params["apm"], real=np.float32)
    full = oracle.crs(g, s.params, "f32", threads=1)
    covered = np.zeros(len(g["cdp_ids"]), bool)
    for (lo, hi), sem, ctr, stk in gathered:
        assert np.array_equal(sem.view(np.uint32), full["str"][lo:hi].view(np.uint32))
        assert np.array_equal(ctr, full["ctr"][lo:hi])
        assert np.array_equal(stk.view(np.uint32), full["stk"][lo:hi].view(np.uint32))
        covered[lo:hi] = True
    assert covered.all()


def test_bench_segments_are_independent_surveys():
    """A multi-GPU bench run gives rank r segment r of the workload: the same
    shapes from another seed, CDP numbers after the earlier segments' and
    coordinates far enough apart that no CRS CDP has a neighbour in another
    segment; segment 0 is the one-GPU workload itself."""
    a = synth.config(3, ncdp=64)
    b = synth.config(3, ncdp=64, segment=1)
    assert np.array_equal(synth.config(3, ncdp=64, segment=0).samples, a.samples)
    assert a.headers["cdp"].max() < b.headers["cdp"].min()
    assert not np.array_equal(a.samples[:10], b.samples[:10])
    fa = np.concatenate([[0], np.cumsum(a.info["fold"])[:-1]])
    fb = np.concatenate([[0], np.cumsum(b.info["fold"])[:-1]])
    both = {k: np.concatenate([a.headers[k][fa], b.headers[k][fb]]) for k in ("gx", "gy", "sx", "sy", "scalco")}
    mx, my = shard.first_trace_midpoints(both)
    lists = shard.neighbours_of(mx, my, a.params["apm"], range(len(mx)))
    n = len(fa)
    assert all(np.all(nb < n) for nb in lists[:n]) and all(np.all(nb >= n) for nb in lists[n:])
