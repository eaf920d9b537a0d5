"""The buoyancy-frequency formula of the device kernel (density differences
formed from temperature and salinity differences with the EOS's polynomial
identities) equals the oracle's direct difference of the two locally
referenced densities; stable stratification gives positive N2."""

import numpy as np

from oracle.models import seos_buoyancy, seos_nsquared


def _difference_form(mask, h, p, S, T):
    A0, B0, L1, L2, M1, M2, NU = 1.6550e-1, 7.6554e-1, 5.9520e-2, 5.4914e-4, 1.4970e-4, 1.1090e-5, 2.4341e-3
    from oracle import oracle as O

    S0, S1, T0, T1 = S[:-1], S[1:], T[:-1], T[1:]
    dT, dS = T1 - T0, S1 - S0
    Ta0, Ta1, Sa0, Sa1 = T0 - 10.0, T1 - 10.0, S0 - 35.0, S1 - 35.0
    zi = 0.5 * (p[:-1] + p[1:])
    dz = 0.5 * (h[:-1] + h[1:])
    drho = (-A0 * dT * (1.0 + 0.5 * L1 * (Ta1 + Ta0) + M1 * zi) + B0 * dS * (1.0 - 0.5 * L2 * (Sa1 + Sa0) - M2 * zi)
            - NU * (dT * Sa1 + Ta0 * dS))
    return np.where(np.asarray(mask)[None] != 0, (-O.GRAVITY / O.RHO0) * drho / dz, np.nan)


def test_difference_form_matches_direct_densities():
    rng = np.random.default_rng(7)
    nz, ny, nx = 12, 5, 6
    h = rng.uniform(0.5, 20.0, (nz, ny, nx))
    p = np.cumsum(h[::-1], axis=0)[::-1] - 0.5 * h  # centre depths, bottom layer deepest
    T = rng.uniform(2.0, 25.0, (nz, ny, nx))
    S = rng.uniform(30.0, 38.0, (nz, ny, nx))
    mask = np.ones((ny, nx), dtype=int)
    mask[0, 0] = 0
    direct = seos_nsquared(mask, h, p, S, T)
    diff = _difference_form(mask, h, p, S, T)
    assert np.isnan(direct[:, 0, 0]).all() and np.isnan(diff[:, 0, 0]).all()
    scale = np.nanmax(np.abs(direct))
    assert np.nanmax(np.abs(direct - diff)) <= 1e-11 * scale


def test_stable_column_has_positive_nsquared():
    nz = 20
    h = np.full((nz, 1, 1), 10.0)
    p = (np.arange(nz)[::-1] * 10.0 + 5.0)[:, None, None]
    T = np.linspace(4.0, 20.0, nz)[:, None, None]  # warmer towards the surface (k = nz-1)
    S = np.full((nz, 1, 1), 35.0)
    NN = seos_nsquared(np.ones((1, 1), dtype=int), h, p, S, T)
    assert (NN > 0).all()
    # direct density difference over the layer spacing, as a check of the sign convention
    r1, _ = seos_buoyancy(S[1:], T[1:], 0.5 * (p[1:] + p[:-1]))
    r0, _ = seos_buoyancy(S[:-1], T[:-1], 0.5 * (p[1:] + p[:-1]))
    assert (r1 < r0).all()


# --- the mixed form's double-float density anomaly, restated on the CPU ---
# float32 operations of numpy round to nearest like the device intrinsics;
# the fused multiply-add is formed from the exact float64 product.
def _f32(x):
    return np.float32(x)


def _fma(a, b, c):
    return _f32(np.float64(a) * np.float64(b) + np.float64(c))


def _fast_sum(s, e):
    h = _f32(s + e)
    return h, _f32(e - _f32(h - s))


def _two_sum(a, b):
    s = _f32(a + b)
    bb = _f32(s - a)
    return s, _f32(_f32(a - _f32(s - bb)) + _f32(b - bb))


def _df_add(x, y):
    s, e = _two_sum(x[0], y[0])
    return _fast_sum(s, _f32(e + _f32(x[1] + y[1])))


def _df_mul(x, y):
    p = _f32(x[0] * y[0])
    e = _fma(x[0], y[0], -p)
    e = _fma(x[0], y[1], _fma(x[1], y[0], e))
    return _fast_sum(p, e)


def _df_const(c):
    hi = _f32(c)
    return hi, _f32(c - np.float64(hi))


def _trunc32(x):
    b = np.array([x], dtype=np.float64).view(np.uint64)[0] & ~np.uint64((1 << 29) - 1)
    return _f32(np.array([b], dtype=np.uint64).view(np.float64)[0])


def _anomaly_df(S, T, z):
    A0, B0, L1, L2, M1, M2, NU = 1.6550e-1, 7.6554e-1, 5.9520e-2, 5.4914e-4, 1.4970e-4, 1.1090e-5, 2.4341e-3
    zh = _trunc32(z)
    zd = (zh, _trunc32(z - np.float64(zh)))
    Ta = _two_sum(_f32(T), _f32(-10.0))
    Sa = _two_sum(_f32(S), _f32(-35.0))
    one = (_f32(1.0), _f32(0.0))
    u = _df_add(one, _df_add(_df_mul(_df_const(0.5 * L1), Ta), _df_mul(_df_const(M1), zd)))
    v = _df_add(_df_mul(_df_const(0.5 * L2), Sa), _df_mul(_df_const(M2), zd))
    v = _df_add(one, (-v[0], -v[1]))
    tA = _df_mul(_df_const(A0), _df_mul(u, Ta))
    tB = _df_mul(_df_const(B0), _df_mul(v, Sa))
    tN = _df_mul(_df_const(NU), _df_mul(Ta, Sa))
    r = _df_add(_df_add((-tA[0], -tA[1]), tB), (-tN[0], -tN[1]))
    return np.float64(r[0]) + np.float64(r[1])


def test_double_float_anomaly_error():
    """The density anomaly rho - 1026 of the mixed form (double-float
    arithmetic from float S and T) against exact rational arithmetic: within
    2e-14 of (1 + |anomaly|) kg m-3, and closer than the FP64 evaluation of
    rho minus 1026, which loses digits to the cancellation."""
    from fractions import Fraction as F

    A0, B0, L1, L2, M1, M2, NU = 1.6550e-1, 7.6554e-1, 5.9520e-2, 5.4914e-4, 1.4970e-4, 1.1090e-5, 2.4341e-3
    rng = np.random.default_rng(3)
    worst_df = worst_64 = 0.0
    for _ in range(400):
        S, T, z = _f32(rng.uniform(0.0, 40.0)), _f32(rng.uniform(-2.0, 32.0)), rng.uniform(0.0, 6000.0)
        Sx, Tx, zx = F(float(S)), F(float(T)), F(z)
        exact = float(-F(A0) * (1 + F(0.5 * L1) * (Tx - 10) + F(M1) * zx) * (Tx - 10)
                      + F(B0) * (1 - F(0.5 * L2) * (Sx - 35) - F(M2) * zx) * (Sx - 35)
                      - F(NU) * (Tx - 10) * (Sx - 35))
        rho64, _ = seos_buoyancy(np.float64(S), np.float64(T), z)
        worst_df = max(worst_df, abs(_anomaly_df(S, T, z) - exact) / (1.0 + abs(exact)))
        worst_64 = max(worst_64, abs((rho64 - 1026.0) - exact) / (1.0 + abs(exact)))
    assert worst_df < 2e-14
    assert worst_df < worst_64
