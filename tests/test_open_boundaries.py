"""Open-boundary collection, masks and point tables on the host, and the
oracle's boundary conditions (no GPU).

The validation cases restate python/tests/test_domain.py:282-336 (outer-edge
boundaries; out-of-range, overlapping, crossing and reversed boundaries) on a
Cartesian domain."""

import numpy as np
import pytest

from getm_gb300.domain import create_cartesian
from getm_gb300.open_boundaries import CLAMPED, FLATHER_ELEV, SPONGE, ZERO_GRADIENT, Side

T2D, T3D = FLATHER_ELEV, ZERO_GRADIENT


def _domain(nx=100, ny=52):
    x = np.linspace(0.0, 1e5, nx)
    y = np.linspace(0.0, 5e4, ny)
    return create_cartesian(x, y, H=10.0, f=1e-4)


def test_outer_edge_boundaries():
    nx, ny = 100, 52
    d = _domain(nx, ny)
    ob = d.open_boundaries
    ob.add_left_boundary("W", 0, 0, ny, T2D, T3D)
    ob.add_top_boundary("N", ny - 1, 1, nx, T2D, T3D)
    ob.add_right_boundary("E", nx - 1, 0, ny - 1, T2D, T3D)
    ob.add_bottom_boundary("S", 0, 1, nx - 1, T2D, T3D)
    T = d.create_grids(10, halox=2, haloy=2, velocity_grids=2)
    assert ob.np == ny + (nx - 1) + (ny - 1) + (nx - 2)
    # every boundary point is a mask-2 T point; the interior stays 1
    assert (T.mask[ob.j, ob.i] == 2).all()
    assert (T.mask == 2).sum() == ob.np
    assert (T.mask[T.haloy + 1:T.haloy + ny - 1, T.halox + 1:T.halox + nx - 1] == 1).all()
    # velocity points just outside the west/east edges are 4, between boundary points 3
    assert (T.ugrid.mask[T.haloy:T.haloy + ny, T.halox - 1] == 4).all()
    assert (T.ugrid.mask == 3).sum() > 0 and (T.vgrid.mask == 3).sum() > 0


def test_invalid_and_adjacent_boundaries():
    nx, ny = 100, 52
    d = _domain(nx, ny)
    ob = d.open_boundaries
    for args in ((-1, 0, 10), (nx, 0, 10), (0, -1, 10), (0, 0, ny + 1)):
        with pytest.raises(AssertionError):
            ob.add_left_boundary("W", *args, T2D, T3D)
    ob.add_right_boundary("E", 10, 10, 11, T2D, T3D)  # a single point
    ob.add_left_boundary("W1", 0, 0, 10, T2D, T3D)
    with pytest.raises(Exception, match="overlaps"):
        ob.add_left_boundary("W2", 0, 9, ny, T2D, T3D)
    ob.add_left_boundary("W2", 0, 10, ny, T2D, T3D)  # directly adjacent
    with pytest.raises(Exception, match="crosses"):
        ob.add_top_boundary("N1", 10, 0, 10, T2D, T3D)
    ob.add_top_boundary("N2", ny - 1, 1, 10, T2D, T3D)
    ob.add_top_boundary("N2", ny - 1, 10, nx, T2D, T3D)
    ob.add_left_boundary("E1", nx - 1, 10, 0, T2D, T3D)  # reversed order
    with pytest.raises(Exception, match="crosses"):
        ob.add_left_boundary("E1", nx - 1, ny - 1, 10, T2D, T3D)
    ob.add_left_boundary("E1", nx - 1, ny - 2, 10, T2D, T3D)
    d.create_grids(10, halox=2, haloy=2, velocity_grids=2)
    reversed_b = [b for b in ob if b.name == "E1"][0]
    assert reversed_b.mstep == -1 and reversed_b.j[0] > reversed_b.j[-1]


def test_boundary_on_land_is_rejected():
    nx, ny = 20, 10
    mask = np.ones((ny, nx), dtype=int)
    mask[3, 0] = 0
    d = create_cartesian(np.arange(nx) * 1e3, np.arange(ny) * 1e3, H=10.0, f=1e-4, mask=mask)
    d.open_boundaries.add_left_boundary("W", 0, 0, ny, T2D, T3D)
    with pytest.raises(Exception, match="on land"):
        d.create_grids(4, halox=2, haloy=2, velocity_grids=2)


def test_mirror_tables():
    from getm_gb300 import workloads

    wl = workloads.tidal_channel()
    T, ob = wl.T, wl.T.open_boundaries
    nx_ = T.nx_
    for name, grid in (("U", T.ugrid), ("V", T.vgrid)):
        src, tgt = getattr(ob, "mirror_" + name)
        assert src.size == tgt.size and np.unique(tgt).size == tgt.size
        # targets are the velocity points just outside (4) or between (3) boundary points
        assert set(np.unique(grid.mask.ravel()[tgt])) <= {3, 4}
    src, tgt = ob.mirror_TU
    assert (T.mask.ravel()[src] == 2).all() and (T.ugrid.mask.ravel()[tgt] == 4).all()
    assert ob.inflow_sign[ob.side == Side.WEST][0] == 1.0 and ob.inflow_sign[ob.side == Side.EAST][0] == -1.0
    assert nx_ == T.nx + 4


def test_oracle_channel_boundary_conditions():
    """Oracle run of the channel: elevations at clamped points equal the
    prescribed tide (clipped), zero-gradient tracer points equal their inward
    neighbours, mirrored transports equal their sources."""
    from getm_gb300 import workloads
    from oracle import models

    wl = workloads.tidal_channel(nx=30, ny=16, nz=4)
    p = wl.params
    s = models.Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    s.temp[...] = np.where(s.T.mask[None] != 0, 10.0 + s.T.zc / 10.0, s.temp)
    s.start(p["timestep"], p["split_factor"])
    for _ in range(3 * p["split_factor"]):
        s.advance()
    ob = wl.T.open_boundaries
    e = [b for b in ob if b.name == "E"][0]
    omega, amp, ph = ob.constituents[0]
    expect = amp[e.start:e.stop] * np.cos(s.time * omega + ph[e.start:e.stop])
    assert np.allclose(s.T.z[e.j, e.i], np.maximum(s.Dmin - s.T.H[e.j, e.i], expect), rtol=0, atol=1e-14)
    w = [b for b in ob if b.name == "W"][0]
    assert np.array_equal(s.temp[:, w.j, w.i], s.temp[:, w.j, w.i + 1])
    src, tgt = ob.mirror_U
    plain = ~np.isin(src, tgt)  # pairs whose source is not itself mirrored
    assert plain.sum() > 0
    assert np.array_equal(s.momentum.U.ravel()[tgt[plain]], s.momentum.U.ravel()[src[plain]])
    assert np.isfinite(s.T.z[s.T.mask != 0]).all()
    assert np.abs(s.T.z[s.T.mask != 0]).max() > 0.1  # the tide came in
