"""Seeded synthetic SU surveys with the shapes of the five benchmark workloads.

The reference ships no dataset (its README names `simple-synthetic.su` and
`fold1000.su`, neither of which is distributed), so every test and benchmark runs
on data made here.  A survey is a list of CDPs (common depth points; common
mid-points for CMP), each with its traces.  Coordinates are integers in
centimetres with scalco = -100, which exercises the reference's negative-scalco
rule (CRS/OpenMP/src/su_trace.cpp:102-107).

Events are 25 Hz Ricker wavelets placed on the CRS traveltime

    t^2 = (t0 + A*dm)^2 + B*dm^2 + C*h^2        (h = half-offset, dm = midpoint
                                                  distance to the block centre)

which reduces to the CMP hyperbola t^2 = t0^2 + C*h^2 for A = B = 0.  Amplitudes are
U[0.5, 1] with a random sign; Gaussian noise has sigma = peak/SNR with SNR = 10 for a
mean peak of 0.75.  All random draws come from numpy's default_rng(seed) (geometry
and events) and default_rng(seed + 1000) (noise).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:  # package-relative when imported as part of the package, plain otherwise
    from . import su as _su
except ImportError:  # pragma: no cover - loaded by file path
    import importlib.util as _ilu
    import os as _os
    _spec = _ilu.spec_from_file_location("semb_su", _os.path.join(_os.path.dirname(__file__), "su.py"))
    _su = _ilu.module_from_spec(_spec)
    _spec.loader.exec_module(_su)

RICKER_HZ = 25.0
NOISE_SIGMA = 0.075


@dataclass
class Survey:
    method: str                 # "cmp" or "crs"
    headers: np.ndarray         # su.HEADER_DTYPE [ntr]
    samples: np.ndarray         # float32 [ntr, ns]
    params: dict                # the reference CLI parameters for this survey
    name: str = ""
    info: dict = field(default_factory=dict)

    @property
    def ntraces(self) -> int:
        return int(self.samples.shape[0])

    @property
    def ns(self) -> int:
        return int(self.samples.shape[1])

    def write(self, path) -> None:
        _su.write_su(path, self.headers, self.samples)

    def cli_args(self, input_path, azimuth: bool = False) -> list:
        """Argument list for cmp-/crs- programs (reference flag names)."""
        p = self.params
        if self.method == "cmp":
            keys = ["c0", "c1", "nc", "aph", "tau"]
        else:
            keys = ["a0", "a1", "na", "b0", "b1", "nb", "c0", "c1", "nc", "aph", "apm", "tau"]
            if azimuth and "azimuth" in p:
                keys.append("azimuth")
        out = []
        for k in keys:
            out += ["-" + k, _fmt(p[k])]
        return out + ["-i", str(input_path)]


def _fmt(v) -> str:
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


def ricker(t: np.ndarray, f: float = RICKER_HZ) -> np.ndarray:
    a = (math.pi * f * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def _build(method, cdp_xy, line_dir, half_offsets, events, block_of_cdp, block_centre,
           ns, dt_us, seed, noise_sigma=NOISE_SIGMA, abs_dm=False, params=None, name=""):
    """Assemble headers and samples.

    cdp_xy [ncdp, 2] midpoint positions (m); line_dir [ncdp, 2] unit source->receiver
    direction; half_offsets: list of arrays (m) per CDP; events: array [nblock, nev, 5]
    of (t0, A, B, C, amp) per block; block_of_cdp [ncdp]; block_centre [nblock, 2]."""
    ncdp = len(cdp_xy)
    fold = np.array([len(h) for h in half_offsets], dtype=np.int64)
    ntr = int(fold.sum())
    cdp_of_tr = np.repeat(np.arange(ncdp), fold)
    h = np.concatenate(half_offsets).astype(np.float64) if ntr else np.zeros(0)
    oi = np.concatenate([np.arange(f) for f in fold]) if ntr else np.zeros(0, np.int64)

    m = cdp_xy[cdp_of_tr]
    d = line_dir[cdp_of_tr]
    s_xy = m - d * h[:, None]
    g_xy = m + d * h[:, None]

    hdr = _su.empty_headers(ntr)
    hdr["tracl"] = np.arange(1, ntr + 1)
    hdr["tracr"] = hdr["tracl"]
    hdr["cdp"] = cdp_of_tr + 1
    hdr["cdpt"] = oi + 1
    hdr["trid"] = 1
    hdr["offset"] = np.rint(2.0 * h).astype(np.int32)
    hdr["scalco"] = -100
    hdr["scalel"] = -100
    hdr["sx"] = np.rint(s_xy[:, 0] * 100.0).astype(np.int32)
    hdr["sy"] = np.rint(s_xy[:, 1] * 100.0).astype(np.int32)
    hdr["gx"] = np.rint(g_xy[:, 0] * 100.0).astype(np.int32)
    hdr["gy"] = np.rint(g_xy[:, 1] * 100.0).astype(np.int32)
    hdr["ns"] = ns
    hdr["dt"] = dt_us

    dt = dt_us * 1e-6
    samples = np.zeros((ntr, ns), dtype=np.float32)
    if noise_sigma > 0 and ntr:
        nrng = np.random.default_rng(seed + 1000)
        chunk = max(1, (1 << 26) // ns)
        for i in range(0, ntr, chunk):
            blk = nrng.standard_normal((min(chunk, ntr - i), ns), dtype=np.float32)
            blk *= np.float32(noise_sigma)
            samples[i:i + chunk] = blk

    if ntr and events is not None and events.shape[1] > 0:
        blk = block_of_cdp[cdp_of_tr]
        # signed distance from the block centre along the line direction
        rel = m - block_centre[blk]
        dm = np.einsum("ij,ij->i", rel, d)
        if abs_dm:
            dm = np.abs(dm)
        half = int(math.ceil(0.06 / dt))
        rows = np.arange(ntr)
        for e in range(events.shape[1]):
            t0, A, B, C, amp = (events[blk, e, k] for k in range(5))
            u = t0 + A * dm
            t2 = u * u + B * dm * dm + C * h * h
            ok = (t2 >= 0) & (amp != 0)
            t = np.sqrt(np.where(ok, t2, 0.0))
            ok &= t < (ns + half) * dt
            r, tt, aa = rows[ok], t[ok], amp[ok]
            i0 = np.floor(tt / dt).astype(np.int64)
            for j in range(-half, half + 1):
                idx = i0 + j
                sel = (idx >= 0) & (idx < ns)
                if not sel.any():
                    continue
                samples[r[sel], idx[sel]] += (aa[sel] * ricker(idx[sel] * dt - tt[sel])).astype(np.float32)

    return Survey(method=method, headers=hdr, samples=samples, params=dict(params or {}), name=name,
                  info={"ncdp": ncdp, "fold": fold})


def _events(rng, nblock, nev, t0_rng, a_rng, b_rng, c_rng):
    ev = np.zeros((nblock, nev, 5))
    ev[..., 0] = rng.uniform(*t0_rng, size=(nblock, nev))
    ev[..., 1] = rng.uniform(*a_rng, size=(nblock, nev)) if a_rng else 0.0
    ev[..., 2] = rng.uniform(*b_rng, size=(nblock, nev)) if b_rng else 0.0
    ev[..., 3] = rng.uniform(*c_rng, size=(nblock, nev))
    ev[..., 4] = rng.uniform(0.5, 1.0, size=(nblock, nev)) * rng.choice([-1.0, 1.0], size=(nblock, nev))
    return ev


CMP_GRID = dict(c0=1.98e-7, c1=1.77e-6)
CRS_GRID = dict(a0=-0.7e-3, a1=0.7e-3, b0=-1e-7, b1=1e-7, c0=1.98e-7, c1=1.77e-6)


def cmp_survey(seed=0, ncmp=200, fold=60, ns=1000, dt_us=2000, nevents=5, nc=101, tau=0.002,
               aph=800, spacing=12.5, half_offsets=None, fold_range=None, hmax=None,
               noise_sigma=NOISE_SIGMA, name="cmp"):
    """CMP line.  Default = the 200-CMP, 60-trace, ns=1000 workload.  With
    `fold_range=(lo, hi)` each CMP's fold is log-uniform in [lo, hi] and its
    half-offsets are U[0, hmax] (the 4096-CMP uneven-fold workload)."""
    rng = np.random.default_rng(seed)
    x = 1000.0 + spacing * np.arange(ncmp)
    cdp_xy = np.stack([x, np.zeros(ncmp)], axis=1)
    line_dir = np.tile([1.0, 0.0], (ncmp, 1))
    if fold_range is not None:
        lo, hi = fold_range
        folds = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), size=ncmp))).astype(int)
        folds = np.clip(folds, lo, hi)
        hofs = [np.sort(rng.uniform(0.0, hmax, size=f)) for f in folds]
    elif half_offsets is not None:
        hofs = [np.asarray(half_offsets, float)] * ncmp
    else:
        hofs = [25.0 + 12.5 * np.arange(fold)] * ncmp
    t_end = 0.9 * ns * dt_us * 1e-6
    ev = _events(rng, ncmp, nevents, (min(0.3, 0.5 * t_end), min(1.8, t_end)), None, None,
                 (CMP_GRID["c0"], CMP_GRID["c1"]))
    # C = 4/v^2 with v ~ U[1500, 4500] m/s
    v = rng.uniform(1500.0, 4500.0, size=(ncmp, nevents))
    ev[..., 3] = 4.0 / (v * v)
    params = dict(CMP_GRID, nc=nc, aph=aph, tau=tau)
    return _build("cmp", cdp_xy, line_dir, hofs, ev, np.arange(ncmp), cdp_xy, ns, dt_us, seed,
                  noise_sigma=noise_sigma, params=params, name=name)


def crs_survey(seed=2, ncdp=500, noffsets=48, ns=1000, dt_us=2000, nevents=4, na=21, nb=21, nc=21,
               tau=0.002, aph=600, apm=50, spacing=12.5, block=16, azimuth=0.0,
               aperture_range=None, line_len=500, noise_sigma=NOISE_SIGMA, abs_dm=False, name="crs"):
    """CRS survey.  Default = the 500-CDP, 48-offset, ns=1000 line.

    With `aperture_range=(lo, hi)` the survey is cut into blocks of `block` CDPs whose
    aperture trace count N (fold x CDPs within apm) is drawn log-uniform in [lo, hi]:
    a block gets a CDP spacing (which sets how many neighbours fall within apm) and a
    fold so that fold * neighbours ~= N.  CDPs are laid on parallel lines of
    `line_len` CDPs spaced far further apart than apm; azimuth 90 lays lines along y."""
    rng = np.random.default_rng(seed)
    az = math.radians(azimuth)
    u = np.array([math.cos(az), math.sin(az)])
    u[np.abs(u) < 1e-12] = 0.0
    perp = np.array([-u[1], u[0]])
    if aperture_range is None:
        spacing_cdp = np.full(ncdp, float(spacing))
        hofs = [12.5 + 12.5 * np.arange(noffsets)] * ncdp
        folds = np.full(ncdp, noffsets)
    else:
        lo, hi = aperture_range
        nblk = (ncdp + block - 1) // block
        target = np.exp(rng.uniform(math.log(lo), math.log(hi), size=nblk))
        spacing_cdp = np.empty(ncdp)
        folds = np.empty(ncdp, dtype=int)
        hmax_blk = rng.uniform(min(600.0, 0.5 * aph), float(aph), size=nblk)
        for b in range(nblk):
            n = target[b]
            # spacing -> neighbours within apm (both sides + self); keep clear of the apm boundary
            if n < 200:
                sp = apm * 0.97
            elif n < 600:
                sp = apm / 3.0 * 0.97
            else:
                sp = apm / 12.0 * 0.97
            nn = 2 * int(apm // sp) + 1
            f = int(np.clip(round(n / nn), 2, 400))
            spacing_cdp[b * block:(b + 1) * block] = sp
            folds[b * block:(b + 1) * block] = f
        hofs = []
        for i in range(ncdp):
            b = i // block
            hofs.append(np.sort(rng.uniform(0.0, hmax_blk[b], size=folds[i])))
    # positions: lines of line_len CDPs, along u, separated along perp by 10*apm + 1000 m
    pos = np.zeros((ncdp, 2))
    for start in range(0, ncdp, line_len):
        sl = slice(start, min(ncdp, start + line_len))
        steps = np.concatenate([[0.0], np.cumsum(spacing_cdp[sl][:-1])])
        lid = start // line_len
        pos[sl] = 1000.0 * u[None, :] + steps[:, None] * u[None, :] + (lid * (10.0 * apm + 1000.0) + 1000.0) * perp[None, :]
    line_dir = np.tile(u, (ncdp, 1))
    nblk = (ncdp + block - 1) // block
    blk_of = np.arange(ncdp) // block
    centre = np.stack([pos[blk_of == b].mean(axis=0) for b in range(nblk)])
    t_end = 0.9 * ns * dt_us * 1e-6
    ev = _events(rng, nblk, nevents, (min(0.3, 0.5 * t_end), min(1.8, t_end)), (CRS_GRID["a0"], CRS_GRID["a1"]),
                 (CRS_GRID["b0"], CRS_GRID["b1"]), (CRS_GRID["c0"], CRS_GRID["c1"]))
    params = dict(CRS_GRID, na=na, nb=nb, nc=nc, aph=aph, apm=apm, tau=tau, azimuth=azimuth)
    s = _build("crs", pos, line_dir, hofs, ev, blk_of, centre, ns, dt_us, seed,
               noise_sigma=noise_sigma, abs_dm=abs_dm, params=params, name=name)
    s.info["spacing"] = spacing_cdp
    return s


def config(idx: int, ncdp: int | None = None, segment: int = 0, **kw) -> Survey:
    """The five benchmark workloads (index 0-4), optionally with fewer CDPs.

    segment > 0 gives another, independent stretch of the same survey: the same
    shapes drawn from another seed (seed + 7919 * segment), its CDP numbers after
    the previous segments' and its coordinates 100 km further along x, so that no
    CDP of one segment lies within the midpoint aperture of another's.  A multi-GPU
    run gives segment r to rank r (weak scaling: per-GPU work stays fixed)."""
    if segment:
        base = _config(idx, ncdp, seed_shift=7919 * segment, **kw)
        n = base.info["ncdp"]
        base.headers["cdp"] += n * segment
        shift = np.int32(10_000_000 * segment)   # cm
        for k in ("sx", "gx"):
            base.headers[k] += shift
        base.name += f"-segment{segment}"
        return base
    return _config(idx, ncdp, **kw)


def _config(idx: int, ncdp: int | None = None, seed_shift: int = 0, **kw) -> Survey:
    if idx == 0:
        return cmp_survey(seed=0 + seed_shift, ncmp=ncdp or 200, name="cmp-200x60-ns1000-nc101", **kw)
    if idx == 1:
        return cmp_survey(seed=1 + seed_shift, ncmp=ncdp or 4096, ns=2000, dt_us=2000, nevents=8, nc=256, tau=0.004,
                          aph=3000, fold_range=(12, 240), hmax=3000.0, name="cmp-4096-fold12to240-ns2000-nc256", **kw)
    if idx == 2:
        return crs_survey(seed=2 + seed_shift, ncdp=ncdp or 500, name="crs-500x48-ns1000-21x21x21", **kw)
    if idx == 3:
        return crs_survey(seed=3 + seed_shift, ncdp=ncdp or 20000, ns=1500, dt_us=4000, nevents=6, tau=0.004, aph=2600,
                          apm=150, azimuth=90.0, aperture_range=(50, 2000), block=32,
                          name="crs-20k-ap50to2000-ns1500-21x21x21", **kw)
    if idx == 4:
        return crs_survey(seed=4 + seed_shift, ncdp=ncdp or 100000, ns=1500, dt_us=4000, nevents=6, na=31, nb=31, nc=31,
                          tau=0.004, aph=2600, apm=150, azimuth=90.0, aperture_range=(50, 2000), block=32,
                          name="crs-100k-ap50to2000-ns1500-31x31x31", **kw)
    raise ValueError(f"unknown workload {idx}")
