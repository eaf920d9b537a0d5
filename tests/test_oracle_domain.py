"""Grid construction and masks (set-up shared by the GPU path and the oracle)
against python/tests/test_domain.py:176-234 (test_grid_mapping, the
non-periodic part): a 100 x 52 Cartesian box of uniform depth with a
2-point halo; the closed edges of the supergrid mask, the T, U, V and X masks
in the interior and on the halos, and land values of H and z0b_min set to
the fill value by Grid.freeze."""

import numpy as np

from getm_gb300.domain import FILL_VALUE, create_cartesian

HALO = 2


def test_grid_mapping():
    Lx, Ly = 100e3, 100e3
    nx, ny = 100, 52
    x = np.linspace(-Lx / 2, Lx / 2, nx)
    y = np.linspace(-Ly / 2, Ly / 2, ny)
    domain = create_cartesian(x, y, H=10.0, lat=0.0)
    assert (domain._H == 10.0).all()
    assert (domain._mask == 1).all()
    domain.infer_UVX_masks2()
    m = domain._mask
    assert (m[1:-1, 1:-1] == 1).all()
    assert (m[0, :] == 0).all() and (m[-1, :] == 0).all()
    assert (m[:, 0] == 0).all() and (m[:, -1] == 0).all()

    T = domain.create_grids(1, halox=HALO, haloy=HALO, velocity_grids=2)
    U, V, X = T.ugrid, T.vgrid, T.xgrid

    def values(g):
        return g.mask[HALO:HALO + g.ny, HALO:HALO + g.nx]

    assert (values(T) == 1).all()
    assert (values(U)[:, :-1] == 1).all() and (values(U)[:, -1] == 0).all()
    assert (values(V)[:-1, :] == 1).all() and (values(V)[-1, :] == 0).all()
    xv = values(X)
    assert (xv[1:-1, 1:-1] == 1).all()
    assert (xv[:, 0] == 0).all() and (xv[:, -1] == 0).all() and (xv[0, :] == 0).all() and (xv[-1, :] == 0).all()

    for g in (T, U, V):
        a = g.mask
        assert (a[:, :HALO] == 0).all() and (a[:, HALO + nx:] == 0).all()
        assert (a[:HALO, :] == 0).all() and (a[HALO + ny:, :] == 0).all()
    a = X.mask
    assert (a[:HALO, :] == 0).all() and (a[HALO + ny + 1:, :] == 0).all()
    assert (a[:, :HALO] == 0).all() and (a[:, HALO + nx + 1:] == 0).all()

    for g in (T, U, V, X):
        assert (g.water == ~g.land).all()
        # land values of H and z0b_min are the fill value (Grid.freeze)
        assert (g.H[g.water] == 10).all() and (g.H[g.land] == FILL_VALUE).all()
        assert (g.z0b_min[g.water] == 0).all() and (g.z0b_min[g.land] == FILL_VALUE).all()
