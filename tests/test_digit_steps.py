"""The digit step of the split-precision kernels, restated in numpy float32.

The kernels take five signed 8-bit digits from a float pair (yh, yl), and
carry the pair scaled by 256 so that a step is six operations: d = rint(Yh),
r = Yh − d, B = 256·Yl, S = fl(256·r + B), Yl ← B + fl(256·r − S), Yh ← S.
Because 256·r is exact, each fused multiply-add there is one float32
addition, so numpy reproduces it exactly.  This test checks, on random pairs
and on exact digit boundaries, that the scaled step gives the same digits
(sign of zero included) as the unscaled two-sum step it replaced:
t = 256·yh, d = rint(t), and (yh, yl) ← the two-sum of t − d and 256·yl.
"""
import numpy as np

f32 = np.float32


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _step_unscaled(yh, yl):
    t = yh * f32(256)
    d = np.rint(t)
    yh, yl = _two_sum(t - d, yl * f32(256))
    return d, yh, yl


def _step_scaled(Yh, Yl):
    d = np.rint(Yh)
    r = Yh - d
    B = Yl * f32(256)
    r256 = r * f32(256)                   # exact
    S = r256 + B                          # fmaf(r, 256, B)
    Yl = B + (r256 - S)                   # B + fmaf(r, 256, -S)
    return d, S, Yl


def _pairs(n, rng):
    v = rng.uniform(-1, 1, n) * np.exp2(-rng.integers(0, 60, n).astype(np.float64))
    # exact digit boundaries: multiples of 2^-8s and half-way points
    k = rng.integers(0, 5, n // 8)
    v[: n // 8] = (rng.integers(-256, 257, n // 8) + 0.5 * rng.integers(0, 2, n // 8)) * np.exp2(-8.0 * (k + 1))
    hi = v.astype(f32)
    lo = (v - hi.astype(np.float64)).astype(f32)
    return hi, lo


def test_scaled_digit_step_gives_the_digits_of_the_two_sum_step():
    rng = np.random.default_rng(7)
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        yh, yl = _pairs(1 << 20, rng)
        yh, yl = _two_sum(yh, yl)
        Yh, Yl = _two_sum(yh * f32(256), yl * f32(256))
        for _ in range(5):
            d0, yh, yl = _step_unscaled(yh, yl)
            d1, Yh, Yl = _step_scaled(Yh, Yl)
            assert np.array_equal(d0, d1)
            assert np.array_equal(np.signbit(d0), np.signbit(d1))
            assert np.all(np.abs(d0) <= 256)


def test_accumulator_split_by_add_subtract_equals_rint():
    """The digit GEMM's drain moves the nearest multiple of 2^12 of each FP32
    accumulator value v (an integer, |v| < 2^24) into a register accumulator.
    It rounds by two additions, (v + 1.5·2^35) − 1.5·2^35: v + 1.5·2^35 lies in
    [2^35, 2^36), where the float32 spacing is 2^12, so the first addition
    rounds v to that spacing (ties to even) and the second is exact.  Checked
    against rint(v·2^-12)·2^12 on random integers, on every tie and on the
    range ends."""
    rng = np.random.default_rng(7)
    v = rng.integers(-(1 << 24) + 1, 1 << 24, size=2_000_000).astype(f32)
    ties = (np.arange(-(1 << 12), 1 << 12, dtype=np.int64) * 4096 + 2048)
    ends = np.array([0, 1, -1, 2047, 2048, 2049, -2048, (1 << 24) - 1, -(1 << 24) + 1], dtype=np.int64)
    v = np.concatenate([v, ties.astype(f32), ends.astype(f32)])
    c = f32(1.5 * 2.0 ** 35)
    hh = (v + c) - c
    assert np.array_equal(hh, np.rint(v * f32(1.0 / 4096)) * f32(4096))
    r = v - hh
    assert np.all(np.abs(r) <= 2048) and np.array_equal(hh + r, v)
