"""The cell rule of the grid neighbour search (csrc/neighbours.cu), restated in numpy:
every CDP pair that the reference's float test accepts, (dx*dx + dy*dy <= apm*apm in
float, CRS/OpenMP/src/su_gather.cpp:70-87), lies in neighbouring cells (at most one
cell apart in x and in y), so scanning the 3 x 3 cells around a CDP finds every
neighbour.  Checked on random layouts at large coordinates and on pairs placed at the
acceptance boundary."""
import numpy as np
import pytest


def cell_of(v, inv_side):
    c = np.floor(v.astype(np.float64) * inv_side)
    return np.clip(c, -(2 ** 30 - 2), 2 ** 30 - 2).astype(np.int64)


def accepted(xi, yi, xj, yj, apm):
    lim = np.float32(np.int32(apm) * np.int32(apm))
    dx = (xj - xi).astype(np.float32)
    dy = (yj - yi).astype(np.float32)
    return (dx * dx + dy * dy).astype(np.float32) <= lim


@pytest.mark.parametrize("apm,origin,spread", [(50, 0.0, 400.0), (25, 6.1e5, 300.0), (120, -3.3e6, 2000.0),
                                              (1, 1.0e5, 8.0), (0, 12.0, 2.0)])
def test_accepted_pairs_are_in_neighbouring_cells(apm, origin, spread):
    rng = np.random.default_rng(apm + 7)
    n = 1500
    x = (origin + rng.uniform(-spread, spread, n)).astype(np.float32)
    y = (origin + rng.uniform(-spread, spread, n)).astype(np.float32)
    # pairs at the boundary: j at distance apm from i along random directions, nudged
    # by one float ulp either way
    k = 300
    th = rng.uniform(0, 2 * np.pi, k)
    xb = (x[:k].astype(np.float64) + apm * np.cos(th)).astype(np.float32)
    yb = (y[:k].astype(np.float64) + apm * np.sin(th)).astype(np.float32)
    up = rng.integers(0, 2, size=k).astype(bool)
    xb = np.nextafter(xb, np.where(up, np.float32(np.inf), np.float32(-np.inf)))
    x = np.concatenate([x, xb])
    y = np.concatenate([y, yb])
    side = (apm if apm > 0 else 1.0) * (1.0 + 1.0 / 1024.0)
    inv = 1.0 / side
    cx, cy = cell_of(x, inv), cell_of(y, inv)
    ok = accepted(x[:, None], y[:, None], x[None, :], y[None, :], apm)
    if apm > 0:
        assert ok.sum() > len(x)   # more than the self pairs
    far = (np.abs(cx[:, None] - cx[None, :]) > 1) | (np.abs(cy[:, None] - cy[None, :]) > 1)
    assert not np.any(ok & far)
