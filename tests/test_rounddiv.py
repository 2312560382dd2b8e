"""The exact offset rounding of the depth plugins (pd_plugins.cuh RoundDiv /
OffsetConst): sign(u)*floor((2|u|+d)/(2d)) via a multiply-high by
m = floor(2^(31+s)/(2d)) + 1, s = floor(log2 2d), must equal
(int)roundf((float)u / (float)d) for |u| <= 2^21 and every depth d in [1, 65535]."""
import numpy as np


def multiplier(d):
    M = 2 * d.astype(np.uint64)
    s = np.floor(np.log2(M.astype(np.float64))).astype(np.uint64)
    return (np.left_shift(np.uint64(1), np.uint64(31) + s) // M + 1).astype(np.uint64), s


def fast_round(u, d):
    m, s = multiplier(d)
    assert np.all(m < 2**32)
    a = np.abs(u).astype(np.uint64)
    n = 2 * a + d.astype(np.uint64)
    q = ((n * m) >> np.uint64(32)) >> (s - np.uint64(1))
    return np.where(u < 0, -q.astype(np.int64), q.astype(np.int64))


def float_round(u, d):
    q = (u.astype(np.float32) / d.astype(np.float32)).astype(np.float32).astype(np.float64)
    return np.trunc(q + np.copysign(0.5, q)).astype(np.int64)  # roundf: exact in float64


def test_every_depth_at_rounding_boundaries():
    d = np.arange(1, 65536, dtype=np.int64)
    for k in (0, 1, 2, 3, 7, 37, 75, 1000):
        for delta in (-1, 0, 1):
            # numerators around the half-integer k + 1/2 and the integer k
            for u0 in ((2 * k + 1) * d // 2 + delta, k * d + delta):
                u = np.clip(u0, -(2**21), 2**21)
                for sign in (1, -1):
                    uu = sign * u
                    assert np.array_equal(fast_round(uu, d), float_round(uu, d))


def test_random_offsets():
    rng = np.random.default_rng(0)
    u = rng.integers(-(2**21), 2**21 + 1, size=2_000_000)
    d = rng.integers(1, 65536, size=2_000_000)
    assert np.array_equal(fast_round(u, d), float_round(u, d))
    u = rng.integers(-60000, 60001, size=2_000_000)
    d = rng.integers(700, 4200, size=2_000_000)
    assert np.array_equal(fast_round(u, d), float_round(u, d))
