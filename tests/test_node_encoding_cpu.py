"""Arithmetic contract of the 8-wide node's plane encoding (CPU).

The BVH collapse stores each quantised child plane q (0..255, in quanta 2^e from the node origin) as
the IEEE half 0x5C00 | q, and the traversal decodes it with one half-to-float conversion and one fused
multiply-add, t = fma(256 + q / 4, 4 s, a - 1024 s) with s = 2^e / d.  These checks pin the two facts
the kernels rely on: the half is exactly 256 + q / 4 for every byte, and the decoded plane distance
stays within 2^-24 (|a| + 2^10 |s|) of a + q s, inside the build's one-quantum slack.
"""
import numpy as np


def test_half_encoding_is_exact_for_every_byte():
    q = np.arange(256, dtype=np.uint16)
    h = (np.uint16(0x5C00) | q).view(np.float16)
    np.testing.assert_array_equal(h.astype(np.float64), 256.0 + q / 4.0)
    np.testing.assert_array_equal(h.astype(np.float32).astype(np.float64), 256.0 + q / 4.0)
    # an empty slot (lo 255, hi 0) decodes to lo > hi, so no ray enters it
    assert h[255].astype(np.float32) > h[0].astype(np.float32)


def test_plane_distance_error_bound():
    rng = np.random.default_rng(7)
    n = 200_000
    q = rng.integers(0, 256, n).astype(np.float64)
    e = rng.integers(-20, 12, n)
    inv_d = rng.uniform(-1e3, 1e3, n) * np.where(rng.random(n) < 0.5, 1e-3, 1.0)
    s = np.ldexp(1.0, e) * inv_d                      # quantum / d, as the kernel forms it (exact power of 2 times 1/d)
    s32 = s.astype(np.float32).astype(np.float64)
    a = rng.uniform(-1e4, 1e4, n).astype(np.float32).astype(np.float64)
    c = (a - 1024.0 * s32).astype(np.float32).astype(np.float64)          # per-node constant, rounded once
    v = 256.0 + q / 4.0
    t = (v * (4.0 * s32) + c).astype(np.float32).astype(np.float64)      # one rounding, as the FFMA
    exact = a + q * s32
    bound = 2.0 ** -24 * (np.abs(a) + 2.0 ** 10 * np.abs(s32)) + 2.0 ** -24 * np.abs(exact) + 1e-300
    assert np.all(np.abs(t - exact) <= 2.0 * bound)
