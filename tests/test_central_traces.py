"""The identity behind the CRS search variant that shares the central traces' sums over
A and B (csrc/pipe_kernel.cuh, central_add): for a trace at zero midpoint distance
(|dm| = dm^2 = 0) the batched kernel's FP32 traveltime of an item, restated here in
numpy with single roundings for each fused multiply-add,

    u0 = fma(A, |dm|, t0),  q0 = fma(u0, u0, C * h),  t^2 = fma(B, dm^2, q0),

equals fma(t0, t0, C * h) bit for bit whatever A and B, so such a trace adds the same
window numerators, energy and in-range count to every (A, B) of one C."""
import numpy as np

F = np.float32


def fma32(a, b, c):
    # a*b is exact in double for float operands; one rounding to float after the add
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(F)


def test_zero_midpoint_distance_makes_the_traveltime_independent_of_a_and_b():
    rng = np.random.default_rng(3)
    n = 200000
    t0 = rng.integers(0, 4000, size=n).astype(F)                          # sample units
    c = (rng.uniform(1.98e-7, 1.77e-6, size=n) * 250.0 ** 2).astype(F)   # C in samples^2/m^2
    h = rng.uniform(0.0, 1300.0 ** 2, size=n).astype(F)                  # squared half-offset
    a = rng.uniform(-0.7e-3, 0.7e-3, size=n).astype(F) * F(250.0)
    b = rng.uniform(-1e-7, 1e-7, size=n).astype(F) * F(250.0 ** 2)
    a[:100] = F(0.0)
    b[100:200] = -F(0.0)
    zero = np.zeros(n, F)
    u0 = fma32(a, zero, t0)
    q0 = fma32(u0, u0, (c * h).astype(F))
    t2 = fma32(b, zero, q0)
    shared = fma32(t0, t0, (c * h).astype(F))
    assert np.array_equal(u0.view(np.uint32), t0.view(np.uint32))
    assert np.array_equal(t2.view(np.uint32), shared.view(np.uint32))
