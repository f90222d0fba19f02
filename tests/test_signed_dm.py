"""The signed midpoint displacement (SEMB_DM_SIGNED), CPU: the oracle's signed branch
against a direct numpy FP64 evaluation of the CRS operator with dm projected on the
azimuth.  The reference has no signed operator, so this pins the oracle's branch to
the definition itself."""
import numpy as np
import pytest

import oracle
import synth


def _numpy_crs_signed(g, params):
    """FP64 CRS search with dm = (mx - mx0) cos(az) + (my - my0) sin(az), following
    the operator of CRS/OpenMP/src/main.cpp:209-285 otherwise (window, validity,
    semblance, argmax from 0 with the lowest index on ties)."""
    sc = g["scalco"].astype(np.float64)   # the scalco rule in double, as the FP64 build
    fs = np.where(sc == 0, 1.0, np.where(sc < 0, 1.0 / np.where(sc == 0, 1.0, sc), sc))
    gx, gy, sx, sy = (g[k].astype(np.float64) for k in ("gx", "gy", "sx", "sy"))
    mx, my = (gx + sx) * fs * 0.5, (gy + sy) * fs * 0.5
    hx, hy = (gx - sx) * fs, (gy - sy) * fs
    h = 0.25 * (hx * hx + hy * hy) / 1e6
    az = np.deg2rad(params["azimuth"])
    ca, sa = np.cos(az), np.sin(az)
    ns, dt = g["ns"], g["dt_us"] / 1e6
    idt = 1.0 / dt
    tau = max(int(params["tau"] * idt), 0)
    w = 2 * tau + 1
    na, nb, nc = params["na"], params["nb"], params["nc"]
    A = params["a0"] + (params["a1"] - params["a0"]) * (1.0 / na) * np.arange(na)
    B = params["b0"] + (params["b1"] - params["b0"]) * (1.0 / nb) * np.arange(nb)
    C = params["c0"] * 1e6 + (params["c1"] * 1e6 - params["c0"] * 1e6) * (1.0 / nc) * np.arange(nc)
    pa, pb, pc = (x.ravel() for x in np.meshgrid(A, B, C, indexing="ij"))
    end = g["ntraces_by_cdp_id"]
    start = np.concatenate([[0], end[:-1]])
    ncdp = len(end)
    ctr = np.zeros((ncdp, ns), np.int64)
    sem_best = np.zeros((ncdp, ns))
    for i in range(ncdp):
        nbr = g["nbr"][g["nbr_off"][i]:g["nbr_off"][i + 1]]
        tr = np.concatenate([np.arange(start[j], end[j]) for j in nbr])
        f0 = start[i]
        m = (mx[tr] - mx[f0]) * ca + (my[tr] - my[f0]) * sa
        s = g["samples"][tr].astype(np.float64)
        for t0 in range(ns):
            T = dt * t0
            t2 = (T + pa[:, None] * m[None, :]) ** 2 + pb[:, None] * (m * m)[None, :] + pc[:, None] * h[tr][None, :]
            t = np.where(t2 < 0, -1.0, np.sqrt(np.maximum(t2, 0.0))) * idt
            it = np.floor(t).astype(np.int64)
            x = t - it
            ok = (t >= 0) & (it - tau >= 0) & (it + tau + 1 < ns)
            M = ok.sum(1)
            err = (~ok).sum(1)
            num = np.zeros((len(pa), w))
            den = np.zeros(len(pa))
            for j in range(w):
                k = np.clip(it - tau + j, 0, ns - 2)
                rows = np.arange(len(tr))[None, :]
                v = (s[rows, k + 1] - s[rows, k]) * x + s[rows, k]
                v = np.where(ok, v, 0.0)
                num[:, j] = v.sum(1)
                den += (v * v).sum(1)
            valid = (den > 1e-13) & (M > 0) & (err < 2)
            sem = np.where(valid, (num ** 2).sum(1) / np.where(valid, den * M, 1.0), 0.0)
            best, bi = 0.0, 0
            for q in range(len(pa)):
                if sem[q] > best:
                    best, bi = sem[q], q
            ctr[i, t0], sem_best[i, t0] = bi, best
    return ctr, sem_best


def test_oracle_signed_branch_matches_numpy_fp64():
    s = synth.crs_survey(seed=41, ncdp=4, noffsets=6, ns=80, dt_us=4000, na=3, nb=2, nc=3, tau=0.004,
                         azimuth=30.0, line_len=4)
    p = dict(s.params)
    g = oracle.gather(s.headers, s.samples, "crs", p["aph"], p["apm"], real=np.float64)
    ref = oracle.crs(g, p, "f64", dm_signed=True)
    ctr, sem = _numpy_crs_signed(g, p)
    np.testing.assert_allclose(ref["str"], sem, rtol=1e-9, atol=1e-12)
    assert np.array_equal(ref["ctr"], ctr)
    # the signed operator is not the reference's |dm| operator on this geometry
    absr = oracle.crs(g, p, "f64")
    assert not np.allclose(absr["str"], ref["str"])
