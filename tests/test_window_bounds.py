"""The planner's per-trace window bounds (trace_window in csrc/semb_kernels.cuh),
restated in numpy float32, against the traveltimes the batched kernel's items compute
(sample units, FP32 with fused multiply-adds).  The check-free path of the batched
search relies on three properties, checked here on random passes:

* a trace classified "every item in range" has tau <= floor(t) <= ns - tau - 2 for
  every (t0, candidate) item of the task and pass;
* a trace left out of the chunk has no item in range;
* every in-range item's window [floor(t) - tau, floor(t) + tau + 1] lies inside the
  staged window [lo, hi]."""
import numpy as np
import pytest

F = np.float32
KTB, KMARGIN = 32, 2


def f32(x):
    return np.asarray(x, dtype=np.float64).astype(F)


def fma32(a, b, c):
    # a*b is exact in double for float operands; one rounding to float after the add
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def trace_window(method, pb, g, T_lo, T_hi, idt, tau, ns):
    """Returns (keep, lo, hi, inrange) as the device function computes them."""
    if method == "cmp":
        t2min = f32(f32(T_lo * T_lo) + min(f32(pb[4] * g[2]), f32(pb[5] * g[2])))
        t2max = f32(f32(T_hi * T_hi) + max(f32(pb[4] * g[2]), f32(pb[5] * g[2])))
    else:
        am0, am1 = f32(pb[0] * g[0]), f32(pb[1] * g[0])
        ulo, uhi = f32(T_lo + min(am0, am1)), f32(T_hi + max(am0, am1))
        u2lo = F(0) if (ulo <= 0 and uhi >= 0) else min(f32(ulo * ulo), f32(uhi * uhi))
        u2hi = max(f32(ulo * ulo), f32(uhi * uhi))
        t2min = f32(f32(u2lo + f32(pb[2] * g[1])) + f32(pb[4] * g[2]))
        t2max = f32(f32(u2hi + f32(pb[3] * g[1])) + f32(pb[5] * g[2]))
    t2min = f32(t2min - f32(abs(t2min) * F(1e-5)))
    t2max = f32(t2max + f32(abs(t2max) * F(1e-5)))
    if not t2max >= 0:
        if t2max < 0:
            return False, 0, 0, False
        return True, 0, ns - 1, False
    smin = f32(f32(np.sqrt(t2min)) * idt) if t2min > 0 else F(0)
    smax = f32(f32(np.sqrt(t2max)) * idt)
    smin, smax = min(smin, F(ns + 8)), min(smax, F(ns + 8))
    inr = bool(t2min > 0 and smin >= tau + 1 and smax <= ns - tau - 3)
    if smax < tau - 1 or smin > ns - tau:
        return False, 0, 0, False
    lo = max(int(smin) - tau - KMARGIN, 0)
    hi = min(int(smax) + tau + 1 + KMARGIN, ns - 1)
    return lo <= hi, lo, hi, inr


def item_index(method, cand, g, t0, idt64):
    """floor(t) of one item as the batched kernel computes it (None: t^2 < 0)."""
    a, b, c = cand
    s1, s2 = idt64, idt64 * idt64
    ca, cb, cc = f32(a * s1), f32(b * s2), f32(c * s2)
    T = F(t0)
    if method == "cmp":
        t2 = fma32(cc, g[2], f32(T * T))
    else:
        u = fma32(ca, g[0], T)
        t2 = fma32(u, u, fma32(cb, g[1], f32(cc * g[2])))
    if not t2 >= 0:
        return None
    return int(np.floor(f32(np.sqrt(np.float64(t2)))))


@pytest.mark.parametrize("method,signed", [("cmp", False), ("crs", False), ("crs", True)])
def test_window_classification_is_safe(method, signed):
    rng = np.random.default_rng({"cmp": 1, "crs": 2}[method] + 10 * signed)
    checked_in = checked_out = 0
    for _ in range(400):
        ns = int(rng.integers(40, 3000))
        dt = float(rng.choice([0.001, 0.002, 0.004]))
        tau = int(rng.integers(0, 8 if method == "cmp" else 3))
        idt = F(1.0) / F(dt)
        idt64 = 1.0 / float(F(dt))
        edge = rng.random() < 0.5   # a task at either end of the record, small offsets
        t0s = int(rng.integers(0, (ns - 1) // KTB + 1)) * KTB
        if edge:
            t0s = int(rng.choice([0, ((ns - 1) // KTB) * KTB, max(0, ((ns - 1) // KTB - 1) * KTB)]))
        T_lo = f32(F(dt) * F(t0s))
        T_hi = f32(F(dt) * F(min(t0s + KTB - 1, ns - 1)))
        # a pass of candidates and its bounds (float grid values, as the plan stores them)
        k = 7
        if method == "cmp":
            c = f32(rng.uniform(2e-7, 2e-6, k) * 1e6)
            cands = [(0.0, 0.0, float(x)) for x in c]
            pb = [F(0), F(0), F(0), F(0), c.min(), c.max()]
            g = (F(0), F(0), f32(rng.uniform(0, 2.5) * (1e-4 if edge else 1.0)))
        else:
            a = f32(rng.uniform(-1e-3, 1e-3, k))
            b = f32(rng.uniform(-1e-6, 1e-6, k))
            c = f32(rng.uniform(-2e-7, 2e-6, k) * 1e6)
            cands = [(float(x), float(y), float(z)) for x, y, z in zip(a, b, c)]
            pb = [a.min(), a.max(), b.min(), b.max(), c.min(), c.max()]
            dm = (rng.uniform(-400, 400) if signed else rng.uniform(0, 400)) * (1e-3 if edge else 1.0)
            g = (f32(dm), f32(dm * dm), f32(rng.uniform(0, 1.5) * (1e-4 if edge else 1.0)))
        keep, lo, hi, inr = trace_window(method, pb, g, T_lo, T_hi, idt, tau, ns)
        for t0 in range(t0s, min(t0s + KTB, ns)):
            for cand in cands:
                it = item_index(method, cand, g, t0, idt64)
                ok = it is not None and tau <= it <= ns - tau - 2
                if inr:
                    assert ok, (ns, tau, t0, cand, g, it)
                    checked_in += 1
                if not keep:
                    assert not ok, (ns, tau, t0, cand, g, it)
                    checked_out += 1
                if keep and ok:
                    assert lo <= it - tau and it + tau + 1 <= hi, (lo, hi, it, tau)
    assert checked_in > 0 and checked_out > 0
