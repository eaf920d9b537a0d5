"""Pins the oracle's advection against the invariants the reference tests
assert (python/tests/test_3d_barotropic.py:259-376): for a flow that satisfies
discrete continuity the Strang-split 3D advection returns the layer
thicknesses to hn (1e-14), conserves the tracer total, keeps a uniform tracer
uniform, and (TVD) keeps a tracer within its initial range."""

import numpy as np
import pytest

from getm_gb300 import workloads
from oracle import oracle as O
from oracle.models import TracerTransport


@pytest.fixture(scope="module")
def wl():
    return workloads.tracer_transport(nx=60, ny=50, nz=10)


def _total(T, c):
    wet = T.mask == 1
    return (c * T.hn / T.iarea)[:, wet].sum()


@pytest.mark.parametrize("scheme", [1, 2, 3, 4, 5, 6])
def test_conservation_and_thickness(wl, scheme):
    m = TracerTransport(wl)
    m.adv = O.Advection(m.T, scheme)
    T = m.T
    c = m.tracers[0]
    tot0 = _total(T, c)
    for _ in range(10):
        m.adv.apply_3d(m.uk, m.vk, m.w, m.dt, c)
        wet = T.mask == 1
        assert np.abs(m.adv.h - T.hn)[:, wet].max() <= 1e-14 * np.abs(T.hn[:, wet]).max()
    assert abs(_total(T, c) - tot0) <= 1e-13 * abs(tot0)


@pytest.mark.parametrize("scheme", [1, 2, 3, 4, 5, 6])
def test_uniform_tracer_stays_uniform(wl, scheme):
    m = TracerTransport(wl)
    T = m.T
    adv = O.Advection(T, scheme)
    c = np.where(T.mask[None] != 0, 3.5, -2e20) * np.ones((T.nz, 1, 1))
    c = np.ascontiguousarray(c)
    for _ in range(5):
        adv.apply_3d(m.uk, m.vk, m.w, m.dt, c)
    wet = T.mask == 1
    assert np.abs(c[:, wet] - 3.5).max() <= 1e-13


@pytest.mark.parametrize("scheme", [5, 6])
def test_tvd_bounds(wl, scheme):
    m = TracerTransport(wl)
    T = m.T
    adv = O.Advection(T, scheme)
    c = m.tracers[0]
    wet = T.mask == 1
    lo, hi = c[:, wet].min(), c[:, wet].max()
    for _ in range(20):
        adv.apply_3d(m.uk, m.vk, m.w, m.dt, c)
    assert c[:, wet].min() >= lo - 1e-12
    assert c[:, wet].max() <= hi + 1e-12


def test_limiter_values():
    """limiters.h:1-44 at a few ratios (cfl = 0.5)."""
    lim = O._lib.oracle_limiter
    # superbee: max(min(2r,1), min(r,2))
    assert lim(5, 0.25, 0.5) == 0.5 and lim(5, 0.75, 0.5) == 1.0 and lim(5, 1.5, 0.5) == 1.5 and lim(5, 3.0, 0.5) == 2.0
    # MUSCL: min(2r, (1+r)/2, 2)
    assert lim(2, 0.2, 0.5) == 0.4 and lim(2, 1.0, 0.5) == 1.0 and lim(2, 5.0, 0.5) == 2.0
    # SPLMAX13: min(2r, max(1+2r, 2+r)/3, 2)
    assert lim(4, 0.1, 0.5) == 0.2 and lim(4, 10.0, 0.5) == 2.0
    # upstream
    assert lim(6, 1.0, 0.5) == 0.0
    # P2_PDM at cfl = 0.5: x = 0, limiter = min(2r/(cfl+1e-10), 0.5 + 0.5r, 2/(1-cfl))
    assert abs(lim(3, 1.0, 0.5) - 1.0) < 1e-15
    # HSIMT never negative
    assert lim(1, 0.01, 0.9) >= 0.0


def test_vertical_substep_count():
    """w3d takes ceil(max cfl) sub-steps (template :298-312); the Courant
    number comes from w_var while the thickness change comes from w, so with
    w = 0 the thickness stays fixed and no restart happens."""
    wl2 = workloads.tracer_transport(nx=20, ny=16, nz=6)
    m = TracerTransport(wl2)
    T = m.T
    w = np.zeros((T.nz + 1, T.ny_, T.nx_))
    w_var = np.zeros_like(w)
    hmin = np.where(T.mask == 1, T.hn.min(axis=0), np.inf).min()
    w_var[1:-1] = 2.5 * hmin / m.dt
    c = np.ascontiguousarray(m.tracers[0])
    h = np.ascontiguousarray(T.hn.copy())
    it = O._lib.oracle_advection_w_calculate(5, T.imin, T.imax, T.jmin, T.jmax, T.nz, 2, 2, O._p(w), O._p(w_var),
                                             O._pi(T.mask), O.c_double(m.dt), O._p(h), O._p(c))
    assert it == 3
    assert np.array_equal(h, T.hn)
