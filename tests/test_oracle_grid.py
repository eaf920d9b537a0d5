"""Pins grid construction and the oracle's staggered interpolation and
Coriolis terms against python/tests/test_grid.py:11-80 (exact T->U/V/UU/VV,
1e-14 T->X/UV) and python/tests/test_coriolis.py:14-80 (f u recovered exactly,
halved at the closed edges)."""

import numpy as np
import pytest

from getm_gb300.domain import coriolis, create_cartesian
from oracle import models
from oracle import oracle as O

TOLERANCE = 1e-14


def _grids():
    dom = create_cartesian(np.linspace(0.0, 10000.0, 101), np.linspace(0.0, 10000.0, 100), H=100.0, f=0.0)
    return O.make_grids(dom.create_grids(30, halox=2, haloy=2, velocity_grids=2))


@pytest.mark.parametrize("nlev", [None, 30, 31])
def test_interpolation(nlev):
    T = _grids()
    rng = np.random.default_rng(1)
    shape = (T.ny_, T.nx_) if nlev is None else (nlev, T.ny_, T.nx_)
    t = rng.random(shape)

    def on(g):
        s = (g.ny_, g.nx_) if nlev is None else (nlev, g.ny_, g.nx_)
        return np.full(s, np.nan)

    u = O.interpolate(T, T.ugrid, t, on(T.ugrid))
    assert (u[..., :, :-1] == 0.5 * (t[..., :, :-1] + t[..., :, 1:])).all()
    v = O.interpolate(T, T.vgrid, t, on(T.vgrid))
    assert (v[..., :-1, :] == 0.5 * (t[..., :-1, :] + t[..., 1:, :])).all()
    x = O.interpolate(T, T.xgrid, t, on(T.xgrid))
    xc = 0.25 * (t[..., :-1, :-1] + t[..., :-1, 1:] + t[..., 1:, :-1] + t[..., 1:, 1:])
    assert np.abs(x[..., 1:-1, 1:-1] - xc).max() < TOLERANCE
    uu = O.interpolate(T, T.ugrid.ugrid, t, on(T.ugrid.ugrid))
    assert (uu[..., :-1] == t[..., 1:]).all()
    vv = O.interpolate(T, T.vgrid.vgrid, t, on(T.vgrid.vgrid))
    assert (vv[..., :-1, :] == t[..., 1:, :]).all()
    uv = O.interpolate(T.ugrid, T.ugrid.vgrid, u, on(T.ugrid.vgrid))
    vu = O.interpolate(T.vgrid, T.vgrid.ugrid, v, on(T.vgrid.ugrid))
    # U -> UV and V -> VU both average to the same corner value
    assert np.abs(uv[..., :-1, :-1] - xc[..., :, :]).max() < TOLERANCE
    assert np.abs(vu[..., :-1, :-1] - xc[..., :, :]).max() < TOLERANCE
    xr = rng.random(x.shape)
    t2 = O.interpolate(T.xgrid, T, xr, on(T))
    tc = 0.25 * (xr[..., :-1, :-1] + xr[..., :-1, 1:] + xr[..., 1:, :-1] + xr[..., 1:, 1:])
    assert np.abs(t2[..., :, :] - tc[..., : t2.shape[-2], : t2.shape[-1]]).max() < TOLERANCE


@pytest.mark.parametrize("lat", [-50.0, 0.0, 20.0])
@pytest.mark.parametrize("u,v", [(-5.0, 5.0), (5.0, 5.0), (0.0, -5.0)])
def test_coriolis(lat, u, v):
    H = 100.0
    x = np.linspace(0, 100000, 100)
    y = np.linspace(0, 100000, 100)
    dom = create_cartesian(x, y, interfaces=True, lat=lat, H=H)
    T = O.make_grids(dom.create_grids(30, halox=2, haloy=2, velocity_grids=2))
    m = models.Momentum()
    m.initialize(T, 4, 5)
    U, V = T.ugrid, T.vgrid
    m.U[...] = np.where(U.mask != 0, u * H, 0.0)
    m.V[...] = np.where(V.mask != 0, v * H, 0.0)
    m.coriolis(U, m.U, V, m.corV, True)
    m.coriolis(V, m.V, U, m.corU, False)
    f = float(coriolis(lat))
    assert (T.cor[T.interior[1:]] == f).all()
    assert (U.cor[U.interior[1:]] == f).all()
    fu = (m.corV / V.H)[V.interior[1:]]
    fv = (m.corU / U.H)[U.interior[1:]]
    assert (fu[:-1, 1:-1] == -f * u).all()
    assert (fu[:-1, 0] == -0.5 * f * u).all()
    assert (fu[:-1, -1] == -0.5 * f * u).all()
    assert (fv[1:-1, :-1] == f * v).all()
    assert (fv[0, :-1] == 0.5 * f * v).all()
    assert (fv[-1, :-1] == 0.5 * f * v).all()
    if u == v:
        assert (fu == -fv.T).all()


def test_mask_closure():
    """U/V points next to land and X points touching land are closed
    (python/pygetm/domain.py:918-941, python/pygetm/core.py:380-390)."""
    rng = np.random.default_rng(3)
    mask = (rng.random((20, 30)) > 0.3).astype(int)
    dom = create_cartesian(np.arange(30) * 1000.0, np.arange(20) * 1000.0, mask=mask, H=20.0, f=0.0)
    T = dom.create_grids(5, halox=2, haloy=2, velocity_grids=2)
    tm = T.mask
    assert ((T.ugrid.mask[:, :-1] == 0) | ((tm[:, :-1] != 0) & (tm[:, 1:] != 0))).all()
    assert ((T.vgrid.mask[:-1, :] == 0) | ((tm[:-1, :] != 0) & (tm[1:, :] != 0))).all()
    X = T.xgrid.mask
    ok = (tm[:-1, :-1] != 0) & (tm[:-1, 1:] != 0) & (tm[1:, :-1] != 0) & (tm[1:, 1:] != 0)
    assert ((X[1:-1, 1:-1] == 0) | ok).all()
    # advection grids of U: UU points closed unless both U neighbours are open
    um, uu = T.ugrid.mask, T.ugrid.ugrid.mask
    assert ((uu[:, :-1] == 0) | ((um[:, :-1] != 0) & (um[:, 1:] != 0))).all()
    # land fill
    assert (T.H[tm == 0] == -2e20).all()
    assert np.allclose(T.iarea[T.interior[1:]], 1.0 / T.area[T.interior[1:]])
