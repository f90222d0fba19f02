"""Arithmetic of the batched kernel's w = 3 packed value/difference staging (LAY_PD in
csrc/semb_kernels.cuh), restated in numpy float32: entries (s_k, s_k+2, d_k, d_k+2) with
d_j = s_j+1 - s_j; window samples 0 and 2 are fma(d, x, s); sample 1 rebuilds
s_1 = s_0 + d_0 and d_1 = s_2 - s_1 before its fma.  The interpolated window values
must stay within a few float roundings of the exact linear interpolation of the
stored (FP16-quantised) samples, for any weight x in [0, 1)."""
import numpy as np

F = np.float32


def fma32(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def test_packed_value_difference_window_is_the_interpolation():
    rng = np.random.default_rng(5)
    n = 200000
    scale = F(0.37)
    # FP16 store times an FP32 per-trace scale, as the conversion stage expands it
    s = (rng.standard_normal((n, 4)) * 3000).astype(np.float16).astype(F) * scale
    x = rng.random(n).astype(F)
    d0, d2 = (s[:, 1] - s[:, 0]).astype(F), (s[:, 3] - s[:, 2]).astype(F)
    v0 = fma32(d0, x, s[:, 0])
    v2 = fma32(d2, x, s[:, 2])
    s1 = (s[:, 0] + d0).astype(F)
    v1 = fma32((s[:, 2] - s1).astype(F), x, s1)
    exact = [s[:, j].astype(np.float64) + x.astype(np.float64) * (s[:, j + 1].astype(np.float64) - s[:, j])
             for j in range(3)]
    mag = np.abs(s).max(axis=1).astype(np.float64)
    ulp = mag * 2.0 ** -23
    for got, want in zip((v0, v1, v2), exact):
        assert np.all(np.abs(got.astype(np.float64) - want) <= 4 * ulp)


def test_side_entry_window_w5_is_the_interpolation():
    """w = 5 with side entries (LAY_PD5): main entry (s_0, s_2, d_0, d_2), side entry
    (s_4, d_4); (s_1, s_3) = (s_0, s_2) + (d_0, d_2), (d_1, d_3) = (s_2 - s_1, s_4 - s_3).
    The five window values stay within a few float roundings of the interpolation."""
    rng = np.random.default_rng(6)
    n = 200000
    scale = F(0.61)
    s = (rng.standard_normal((n, 6)) * 3000).astype(np.float16).astype(F) * scale
    x = rng.random(n).astype(F)
    d = [(s[:, j + 1] - s[:, j]).astype(F) for j in range(5)]
    v0 = fma32(d[0], x, s[:, 0])
    v2 = fma32(d[2], x, s[:, 2])
    s1 = (s[:, 0] + d[0]).astype(F)
    s3 = (s[:, 2] + d[2]).astype(F)
    v1 = fma32((s[:, 2] - s1).astype(F), x, s1)
    v3 = fma32((s[:, 4] - s3).astype(F), x, s3)
    v4 = fma32(d[4], x, s[:, 4])
    exact = [s[:, j].astype(np.float64) + x.astype(np.float64) * (s[:, j + 1].astype(np.float64) - s[:, j])
             for j in range(5)]
    ulp = np.abs(s).max(axis=1).astype(np.float64) * 2.0 ** -23
    for got, want in zip((v0, v1, v2, v3, v4), exact):
        assert np.all(np.abs(got.astype(np.float64) - want) <= 4 * ulp)
