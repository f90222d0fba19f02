"""Sharding a survey across ranks (one process per GPU).

The search is independent per CDP, so N GPUs split the CDPs into N contiguous
ranges with no exchange step.  A CMP search needs only the owned CDPs' traces; a
CRS search also needs, read-only, the traces of every CDP within the midpoint
aperture apm of an owned CDP (the halo), which each rank loads itself.  The
neighbour rule is the reference's (CRS/OpenMP/src/su_gather.cpp:70-87): first-trace
midpoints fscalco * (gx + sx) * 0.5 in float, distance^2 <= apm^2 in float.

Ranks weight their ranges by search work (aperture traces x ns x candidates) so a
rank with dense CDPs gets fewer of them.
"""
from __future__ import annotations

import numpy as np


def fscalco(scalco: np.ndarray) -> np.ndarray:
    s = scalco.astype(np.float32)
    out = np.where(scalco == 0, np.float32(1.0), s).astype(np.float32)
    neg = scalco < 0
    out[neg] = np.float32(1.0) / s[neg]
    return out


def first_trace_midpoints(first_hdr: dict) -> tuple[np.ndarray, np.ndarray]:
    """Float midpoints of each CDP's first trace (su_trace::midpoint_x/y)."""
    fs = fscalco(np.asarray(first_hdr["scalco"]))
    gx, sx = np.asarray(first_hdr["gx"], np.int32), np.asarray(first_hdr["sx"], np.int32)
    gy, sy = np.asarray(first_hdr["gy"], np.int32), np.asarray(first_hdr["sy"], np.int32)
    mx = (fs * (gx + sx).astype(np.float32)) * np.float32(0.5)
    my = (fs * (gy + sy).astype(np.float32)) * np.float32(0.5)
    return mx, my


def neighbours_of(mx: np.ndarray, my: np.ndarray, apm: int, cdps) -> list:
    """Neighbour lists (ascending) of the CDPs in `cdps`."""
    lim = np.float32(int(apm) * int(apm))
    out = []
    for i in cdps:
        dx = mx - mx[i]
        dy = my - my[i]
        out.append(np.nonzero((dx * dx + dy * dy) <= lim)[0])
    return out


def split_ranges(weights: np.ndarray, world: int) -> list:
    """Contiguous [lo, hi) CDP ranges with about equal total weight."""
    w = np.asarray(weights, dtype=np.float64)
    n = len(w)
    if world <= 1 or n == 0:
        return [(0, n)]
    cum = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(cum, cum[-1] * r / world)))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, n))
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


class Shard:
    """The part of a linearized gather one rank loads: its owned CDP range plus,
    for CRS, the halo CDPs; `owned_local` are the owned CDPs' indices in the
    shard's own CDP numbering."""

    def __init__(self, cdps: np.ndarray, owned: tuple, owned_local: np.ndarray):
        self.cdps = cdps                  # global CDP indices in the shard, ascending
        self.owned = owned                # (lo, hi) global
        self.owned_local = owned_local    # positions of owned CDPs within self.cdps

    def select(self, cdp_end: np.ndarray, arrays: dict) -> dict:
        """Slice per-trace arrays (and rebuild cdp_end) for the shard's CDPs."""
        starts = np.concatenate([[0], cdp_end[:-1]])
        rows = np.concatenate([np.arange(starts[c], cdp_end[c]) for c in self.cdps])
        out = {k: v[rows] for k, v in arrays.items()}
        folds = cdp_end[self.cdps] - starts[self.cdps]
        out["cdp_end"] = np.cumsum(folds).astype(np.int64)
        return out


def plan_shard(method: str, cdp_end: np.ndarray, first_hdr: dict, apm: int, world: int, rank: int,
               weights: np.ndarray | None = None) -> Shard:
    ncdp = len(cdp_end)
    folds = np.diff(np.concatenate([[0], cdp_end]))
    if method == "crs":
        mx, my = first_trace_midpoints(first_hdr)
    if weights is None:
        if method == "crs":
            weights = np.array([folds[nb].sum() for nb in neighbours_of(mx, my, apm, range(ncdp))], np.float64)
        else:
            weights = folds.astype(np.float64)
    lo, hi = split_ranges(weights, world)[rank]
    owned = np.arange(lo, hi)
    if method == "crs" and hi > lo:
        need = np.unique(np.concatenate(neighbours_of(mx, my, apm, owned) + [owned]))
    else:
        need = owned
    owned_local = np.searchsorted(need, owned)
    return Shard(need, (lo, hi), owned_local)
