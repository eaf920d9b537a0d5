"""The integer-pipe conversions of getm_common.cuh restated on IEEE-754 bit
fields with numpy, against the hardware casts and multiplies: getm_f2d is
the exact float -> double widening, getm_d2f_approx truncates the mantissa
(relative error below 2^-23), and getm_half / getm_quarter give bitwise the
FP64 product with 0.5 / 0.25 wherever they take the integer path."""

import numpy as np


def _f2d(x):
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    e = (b >> 23) & 0xFF
    s = (b >> 31) << 63
    m = (b & 0x7FFFFF) << 29
    de = (e + (1023 - 127)) << 52
    fast = (e != 0) & (e != 0xFF)
    out = np.where(fast, (s | de | m).view(np.float64), np.asarray(x, dtype=np.float32).astype(np.float64))
    return out, fast


def _d2f_approx(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    e = ((b >> 52) & 0x7FF).astype(np.int64) - 1023 + 127
    fast = (e > 0) & (e < 0xFF)
    s = ((b >> 63) << 31).astype(np.uint32)
    m = ((b >> 29) & 0x7FFFFF).astype(np.uint32)
    bits = s | (np.clip(e, 0, 255).astype(np.uint32) << 23) | m
    with np.errstate(over="ignore"):  # the hardware path of out-of-range values
        hw = np.asarray(x).astype(np.float32)
    return np.where(fast, bits.view(np.float32), hw), fast


def _scale_down(x, n):
    b = np.asarray(x, dtype=np.float64).view(np.int64)
    e = (b >> 52) & 0x7FF
    fast = (e > n) & (e < 0x7FF)
    return np.where(fast, (b - (np.int64(n) << 52)).view(np.float64), x * (0.5 if n == 1 else 0.25)), fast


def _sample(rng, n):
    mag = 10.0 ** rng.uniform(-40, 40, n)
    x = np.where(rng.random(n) < 0.5, -mag, mag)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308, 1.0, -3.5])
    return np.concatenate([x, special])


def test_f2d_is_exact_widening():
    rng = np.random.default_rng(1)
    with np.errstate(over="ignore"):  # magnitudes beyond float32 become infinities
        x = _sample(rng, 20000).astype(np.float32)
    got, fast = _f2d(x)
    want = x.astype(np.float64)
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all()
    assert fast.mean() > 0.9


def test_d2f_approx_truncates_within_2_pow_minus_23():
    rng = np.random.default_rng(2)
    x = _sample(rng, 20000)
    got, fast = _d2f_approx(x)
    sel = fast & np.isfinite(x) & (x != 0)
    rel = np.abs(got[sel].astype(np.float64) - x[sel]) / np.abs(x[sel])
    assert rel.max() < 2.0 ** -23
    # truncation: never larger in magnitude than the double
    assert (np.abs(got[sel].astype(np.float64)) <= np.abs(x[sel])).all()


def test_pow2_scale_down_is_the_fp64_product():
    rng = np.random.default_rng(3)
    x = _sample(rng, 20000)
    for n, f in ((1, 0.5), (2, 0.25)):
        got, fast = _scale_down(x, n)
        want = x * f
        same = (got == want) | (np.isnan(got) & np.isnan(want))
        assert same.all()
        assert (np.signbit(got[fast]) == np.signbit(want[fast])).all()
        assert fast.mean() > 0.9
